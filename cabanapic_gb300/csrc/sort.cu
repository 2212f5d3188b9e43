// sort.cu -- counting sort of the particle AoSoA by cell index.
//
// The reference leaves its sort commented out (example/example.cpp:226-228,
// Cabana::sortByKey on the cell slice).  Sorting every few steps keeps a
// warp's particles in one or two cells, which turns the push's 18-coefficient
// gather into a broadcast and lets its deposit reduce within the warp.
//
// Passes (keys are cell indices in [0, num_cells); an out-of-range key sorts
// after all valid ones):
//   1. count:   per-cell particle counts (reductions, no return values)
//   2. scan:    exclusive prefix sum of the counts -> cell offsets
//   3. scatter: each particle takes the next slot of its cell from the offset
//               (atomics with return) and writes perm[slot] = its index
//   4. gather:  particles[d] = copy[perm[d]], member by member (coalesced writes),
//               in two launches of four members each
// Passes 1 and 3 aggregate over the lanes of a warp that share a cell: one
// atomic per cell per 32 particles.  Each warp takes kSortChunks chunks of 32
// particles, with all loads and atomics issued before their results are used.
// The order within a cell depends on atomic arrival order.  The in-place entry
// point gathers from a copy of the list in the scratch; the out-of-place one
// (for callers with two lists) gathers straight into the second list and
// skips that copy.
//
// Look-ahead keys (cpic_sort_particles_ahead_into): the key of a particle is
// the interior cell it reaches after `steps` free-streaming pushes at its
// current momentum (the push's displacement 2 u cdt_d / gamma per step,
// wrapped periodically; ghost and out-of-range cells keep their own key).  A
// list sorted on the cells half a sort interval ahead is in order midway
// through the interval instead of at its start, so the mean spread of a
// warp's 32 particles over cells across the interval is smaller.
#include <cuda_runtime.h>

#include "common.cuh"

namespace cpic {

constexpr int kSortThreads = 256;
constexpr int kSortChunks = 4;  // 32-particle chunks per warp in the count and scatter passes
constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

static inline size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

struct SortPlan {
  size_t counts_off, sums_off, perm_off, copy_off, total;
  int64_t nkeys, nscan_blocks;
};

static SortPlan plan_sort(int64_t n, int64_t num_cells, int prec, int vl) {
  SortPlan p;
  p.nkeys = num_cells + 1;  // last key collects out-of-range cells
  p.nscan_blocks = (p.nkeys + kScanTile - 1) / kScanTile;
  size_t off = 0;
  p.counts_off = off; off += align256(sizeof(int) * (size_t)p.nkeys);
  p.sums_off = off;   off += align256(sizeof(int) * (size_t)p.nscan_blocks);
  p.perm_off = off;   off += align256(sizeof(int) * (size_t)n);
  p.copy_off = off;   off += align256(cpic_particle_list_bytes(n, prec, vl));
  p.total = off;
  return p;
}

// Look-ahead key parameters: k = 2 * steps * cdt_d per axis (offset units per
// unit of u / gamma; a cell is 2 offset units wide); the ghosted row and plane
// extents with their multiply-shift divisors.
template <class R>
struct SortAhead {
  R kx, ky, kz;
  int nx, ny, nz, sx, sy;
  DivMagic dsx, dsy;
};

// Interior index (1..n) reached from index i by a predicted offset f.  The
// offset is clamped to +-(2n - 1) (also NaN, to -(2n - 1)), so the shift lies
// in [1 - n, n] and one correction wraps it periodically; a particle that
// would cross the whole grid takes some cell of it, which any order allows.
template <class R>
__device__ __forceinline__ int ahead_index(int i, R f, int n) {
  const R lim = (R)(2 * n - 1);
  if (!(f >= -lim)) f = -lim;
  if (!(f <= lim)) f = lim;
  int j = i - 1 + (int)floor((f + (R)1) * (R)0.5);
  if (j < 0) j += n;
  if (j >= n) j -= n;
  return j + 1;
}

// Cell key of particle p: out-of-range cells go to the last bucket; lanes
// past the end get distinct negative keys.  AHEAD: the interior cell the
// particle reaches `steps` pushes ahead.
template <class R, int VL, bool AHEAD>
__device__ __forceinline__ int sort_key(const unsigned char* __restrict__ part, int64_t p, int n,
                                        int num_cells, int lane, const SortAhead<R>& a) {
  using L = PLayout<R, VL>;
  if (p >= n) return -1 - lane;
  const int c = __ldg(reinterpret_cast<const int*>(part + L::cell_off(p)));
  R m[6];
  if (AHEAD) {  // loaded with the cell, before any test on it (all loads in flight together)
#pragma unroll
    for (int k = 0; k < 6; ++k) m[k] = __ldg(reinterpret_cast<const R*>(part + L::off(p, k)));
  }
  if ((unsigned)c >= (unsigned)num_cells) return num_cells;
  if (!AHEAD) return c;
  int ix = c, iy, iz;  // RANK_TO_INDEX by multiply-shift division
  iy = div_magic(ix, a.dsx); ix -= iy * a.sx;
  iz = div_magic(iy, a.dsy); iy -= iz * a.sy;
  if (ix < 1 || ix > a.nx || iy < 1 || iy > a.ny || iz < 1 || iz > a.nz) return c;
  const R rg = (R)1 / sqrt((R)1 + (m[3] * m[3] + (m[4] * m[4] + m[5] * m[5])));
  const int jx = ahead_index<R>(ix, m[0] + a.kx * m[3] * rg, a.nx);
  const int jy = ahead_index<R>(iy, m[1] + a.ky * m[4] * rg, a.ny);
  const int jz = ahead_index<R>(iz, m[2] + a.kz * m[5] * rg, a.nz);
  return jx + a.sx * (jy + a.sy * jz);
}

// Groups of equal keys among the warp's lanes: `leader` is the group's first
// lane, `len` its size and `rank` this lane's place in it.  A chunk made of
// one or two runs of equal keys (most chunks of a sorted list) takes a
// shuffle-and-ballot run test; others group with __match_any_sync, which
// keeps one atomic per distinct cell when strays split a cell's run.
__device__ __forceinline__ void key_group(int key, int lane, int& leader, int& len, int& rank) {
  const int left = __shfl_up_sync(kFull, key, 1);
  const unsigned heads = __ballot_sync(kFull, lane == 0 || key != left);
  if (__popc(heads) <= 2) {  // warp-uniform
    const unsigned upto = 0xffffffffu >> (31 - lane);  // lanes 0..lane
    leader = 31 - __clz(heads & upto);
    const unsigned above = heads & ~upto;
    len = (above ? __ffs(above) - 1 : 32) - leader;
    rank = lane - leader;
  } else {
    const unsigned peers = __match_any_sync(kFull, key);
    leader = __ffs(peers) - 1;
    len = __popc(peers);
    rank = __popc(peers & ((1u << lane) - 1u));
  }
}

__device__ __forceinline__ int64_t sort_chunk0() {
  return ((int64_t)blockIdx.x * (kSortThreads / 32) + (threadIdx.x >> 5)) * kSortChunks;
}

// AHEAD: the count pass also parks each key in the cell member of the output
// list (slot p, overwritten by the gather), where the scatter pass reads it
// back instead of recomputing it from the particle's seven members.
template <class R, int VL, bool AHEAD>
__global__ void __launch_bounds__(kSortThreads)
count_kernel(const unsigned char* __restrict__ part, int n, int num_cells, int* __restrict__ counts,
             SortAhead<R> a, unsigned char* __restrict__ key_park) {
  using L = PLayout<R, VL>;
  const int lane = lane_id();
  const int64_t c0 = sort_chunk0();
  int key[kSortChunks];
#pragma unroll
  for (int k = 0; k < kSortChunks; ++k) key[k] = sort_key<R, VL, AHEAD>(part, (c0 + k) * 32 + lane, n, num_cells, lane, a);
#pragma unroll
  for (int k = 0; k < kSortChunks; ++k) {
    int leader, len, rank;
    key_group(key[k], lane, leader, len, rank);
    if (leader == lane && key[k] >= 0) atomicAdd(counts + key[k], len);
    if (AHEAD && key[k] >= 0)
      *reinterpret_cast<int*>(key_park + L::cell_off((c0 + k) * 32 + lane)) = key[k];
  }
}

template <class R, int VL, bool AHEAD>
__device__ __forceinline__ int scatter_key(const unsigned char* __restrict__ part,
                                           const unsigned char* __restrict__ key_park, int64_t p, int n,
                                           int num_cells, int lane) {
  using L = PLayout<R, VL>;
  if (!AHEAD) return sort_key<R, VL, false>(part, p, n, num_cells, lane, SortAhead<R>{});
  if (p >= n) return -1 - lane;
  return *reinterpret_cast<const int*>(key_park + L::cell_off(p));
}

// Block-local exclusive scan of kScanTile ints; returns the tile total.
__device__ int block_exclusive_scan(int* __restrict__ data, int64_t n, int64_t tile0,
                                    int* __restrict__ warp_tot) {
  int v[kScanItems];
  int local = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    const int64_t i = tile0 + (int64_t)threadIdx.x * kScanItems + k;
    v[k] = i < n ? data[i] : 0;
    local += v[k];
  }
  const int lane = lane_id(), w = threadIdx.x >> 5;
  int incl = local;
  for (int o = 1; o < 32; o <<= 1) {
    int t = __shfl_up_sync(kFull, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) warp_tot[w] = incl;
  __syncthreads();
  if (w == 0) {
    int t = warp_tot[lane];
    int s = t;
    for (int o = 1; o < 32; o <<= 1) {
      int u = __shfl_up_sync(kFull, s, o);
      if (lane >= o) s += u;
    }
    warp_tot[lane] = s - t;  // exclusive prefix of the warp totals
    if (lane == 31) warp_tot[32] = s;
  }
  __syncthreads();
  int run = warp_tot[w] + incl - local;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    const int64_t i = tile0 + (int64_t)threadIdx.x * kScanItems + k;
    if (i < n) data[i] = run;
    run += v[k];
  }
  const int total = warp_tot[32];
  __syncthreads();
  return total;
}

__global__ void __launch_bounds__(kScanThreads)
scan_tiles_kernel(int* __restrict__ data, int64_t n, int* __restrict__ sums) {
  __shared__ int warp_tot[33];
  const int total = block_exclusive_scan(data, n, (int64_t)blockIdx.x * kScanTile, warp_tot);
  if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

// One block scans the tile totals, kScanTile at a time with a running carry.
__global__ void __launch_bounds__(kScanThreads)
scan_sums_kernel(int* __restrict__ sums, int64_t nsums) {
  __shared__ int warp_tot[33];
  __shared__ int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int64_t t0 = 0; t0 < nsums; t0 += kScanTile) {
    const int c = carry;
    __syncthreads();
    const int total = block_exclusive_scan(sums, nsums, t0, warp_tot);
    for (int64_t i = t0 + threadIdx.x; i < nsums && i < t0 + kScanTile; i += blockDim.x) sums[i] += c;
    __syncthreads();
    if (threadIdx.x == 0) carry = c + total;
    __syncthreads();
  }
}

__global__ void __launch_bounds__(kScanThreads)
scan_add_kernel(int* __restrict__ data, int64_t n, const int* __restrict__ sums) {
  const int add = sums[blockIdx.x];
  const int64_t t0 = (int64_t)blockIdx.x * kScanTile;
  for (int k = threadIdx.x; k < kScanTile; k += blockDim.x) {
    const int64_t i = t0 + k;
    if (i < n) data[i] += add;
  }
}

// cursor: the cell offsets, advanced as slots are taken.
template <class R, int VL, bool AHEAD>
__global__ void __launch_bounds__(kSortThreads)
scatter_kernel(const unsigned char* __restrict__ part, int n, int num_cells, int* __restrict__ cursor,
               int* __restrict__ perm, const unsigned char* __restrict__ key_park) {
  const int lane = lane_id();
  const int64_t c0 = sort_chunk0();
  int key[kSortChunks], leader[kSortChunks], rank[kSortChunks], base[kSortChunks];
#pragma unroll
  for (int k = 0; k < kSortChunks; ++k)
    key[k] = scatter_key<R, VL, AHEAD>(part, key_park, (c0 + k) * 32 + lane, n, num_cells, lane);
#pragma unroll
  for (int k = 0; k < kSortChunks; ++k) {
    int len;
    key_group(key[k], lane, leader[k], len, rank[k]);
    base[k] = 0;
    if (leader[k] == lane && key[k] >= 0) base[k] = atomicAdd(cursor + key[k], len);
  }
#pragma unroll
  for (int k = 0; k < kSortChunks; ++k) {
    const int b = __shfl_sync(kFull, base[k], leader[k]);
    const int64_t p = (c0 + k) * 32 + lane;
    if (p < n) perm[b + rank[k]] = (int)p;
  }
}

// Members [M0, M1) of the record (7 = the cell index).  The gather runs in
// kGatherPasses launches over disjoint member ranges, so that the source lines
// a pass touches stay in L2 until every destination that shares them has been
// written (a particle that moved by one plane is (nx+2)(ny+2) cells away in
// the list).  Measured on the 128^3 x 64 ppc plasma 20 steps after a sort
// (ms per sort): 1 pass 4.34, 2 passes 3.81, 4 passes 4.45, 8 passes 6.56;
// more passes re-read the permutation once each.
#ifndef CPIC_SORT_GATHER_PASSES
#define CPIC_SORT_GATHER_PASSES 2
#endif
constexpr int kGatherPasses = CPIC_SORT_GATHER_PASSES;
static_assert(kGatherPasses == 1 || kGatherPasses == 2 || kGatherPasses == 4 || kGatherPasses == 8,
              "gather passes: 1, 2, 4 or 8");

template <class R, int VL, int M0, int M1>
__global__ void __launch_bounds__(kSortThreads)
gather_kernel(const unsigned char* __restrict__ src, unsigned char* __restrict__ dst, int n,
              const int* __restrict__ perm) {
  using L = PLayout<R, VL>;
  const int64_t d = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (d >= n) return;
  const int s = perm[d];
#pragma unroll
  for (int m = M0; m < M1; ++m) {
    if (m < 7)
      *reinterpret_cast<R*>(dst + L::off(d, m)) = __ldg(reinterpret_cast<const R*>(src + L::off(s, m)));
    else
      *reinterpret_cast<int*>(dst + L::cell_off(d)) =
          __ldg(reinterpret_cast<const int*>(src + L::cell_off(s)));
  }
}

template <class R, int VL>
static void launch_gather(const unsigned char* src, unsigned char* dst, int n, const int* perm, unsigned blocks,
                          cudaStream_t s) {
  constexpr int W = 8 / kGatherPasses;
  gather_kernel<R, VL, 0, W><<<blocks, kSortThreads, 0, s>>>(src, dst, n, perm);
  if (kGatherPasses > 1) gather_kernel<R, VL, W, 2 * W><<<blocks, kSortThreads, 0, s>>>(src, dst, n, perm);
  if (kGatherPasses > 2) {
    gather_kernel<R, VL, 2 * W, 3 * W><<<blocks, kSortThreads, 0, s>>>(src, dst, n, perm);
    gather_kernel<R, VL, 3 * W, 4 * W><<<blocks, kSortThreads, 0, s>>>(src, dst, n, perm);
  }
  if (kGatherPasses > 4) {
    gather_kernel<R, VL, 4 * W, 5 * W><<<blocks, kSortThreads, 0, s>>>(src, dst, n, perm);
    gather_kernel<R, VL, 5 * W, 6 * W><<<blocks, kSortThreads, 0, s>>>(src, dst, n, perm);
    gather_kernel<R, VL, 6 * W, 7 * W><<<blocks, kSortThreads, 0, s>>>(src, dst, n, perm);
    gather_kernel<R, VL, 7 * W, 8 * W><<<blocks, kSortThreads, 0, s>>>(src, dst, n, perm);
  }
}

// dst == nullptr: in place, through the particle copy in the scratch;
// otherwise src is gathered into dst (src unchanged, no copy).
template <class R, int VL>
static int sort_typed(void* particles, void* dst, int n, int num_cells, const SortPlan& pl,
                      unsigned char* sc, const SortAhead<R>* ahead, cudaStream_t s) {
  int* counts = reinterpret_cast<int*>(sc + pl.counts_off);
  int* sums = reinterpret_cast<int*>(sc + pl.sums_off);
  int* perm = reinterpret_cast<int*>(sc + pl.perm_off);
  unsigned char* copy = sc + pl.copy_off;
  unsigned char* part = static_cast<unsigned char*>(particles);
  const unsigned pb = (unsigned)(((int64_t)n + kSortThreads - 1) / kSortThreads);
  const int64_t warps = ((int64_t)n + 32 * kSortChunks - 1) / (32 * kSortChunks);
  const unsigned cb = (unsigned)((warps + kSortThreads / 32 - 1) / (kSortThreads / 32));
  if (cudaMemsetAsync(counts, 0, sizeof(int) * (size_t)pl.nkeys, s) != cudaSuccess) return CPIC_ECUDA;
  const SortAhead<R> a = ahead ? *ahead : SortAhead<R>{};
  unsigned char* park = static_cast<unsigned char*>(dst);  // look-ahead keys: out-of-place only
  if (ahead && !park) return CPIC_EINVAL;
  if (ahead)
    count_kernel<R, VL, true><<<cb, kSortThreads, 0, s>>>(part, n, num_cells, counts, a, park);
  else
    count_kernel<R, VL, false><<<cb, kSortThreads, 0, s>>>(part, n, num_cells, counts, a, nullptr);
  scan_tiles_kernel<<<(unsigned)pl.nscan_blocks, kScanThreads, 0, s>>>(counts, pl.nkeys, sums);
  scan_sums_kernel<<<1, kScanThreads, 0, s>>>(sums, pl.nscan_blocks);
  scan_add_kernel<<<(unsigned)pl.nscan_blocks, kScanThreads, 0, s>>>(counts, pl.nkeys, sums);
  if (ahead)
    scatter_kernel<R, VL, true><<<cb, kSortThreads, 0, s>>>(part, n, num_cells, counts, perm, park);
  else
    scatter_kernel<R, VL, false><<<cb, kSortThreads, 0, s>>>(part, n, num_cells, counts, perm, nullptr);
  if (dst) {
    launch_gather<R, VL>(part, static_cast<unsigned char*>(dst), n, perm, pb, s);
    return launch_status();
  }
  const size_t bytes = cpic_particle_list_bytes(n, sizeof(R), VL);
  if (cudaMemcpyAsync(copy, part, bytes, cudaMemcpyDeviceToDevice, s) != cudaSuccess) return CPIC_ECUDA;
  launch_gather<R, VL>(copy, part, n, perm, pb, s);
  return launch_status();
}

template <class R>
static SortAhead<R> make_ahead(const cpic_grid* g, const cpic_push_params* prm, int steps) {
  SortAhead<R> a;
  a.kx = (R)(2.0 * steps * prm->cdt_dx);
  a.ky = (R)(2.0 * steps * prm->cdt_dy);
  a.kz = (R)(2.0 * steps * prm->cdt_dz);
  a.nx = (int)g->nx; a.ny = (int)g->ny; a.nz = (int)g->nz;
  a.sx = a.nx + 2;
  a.sy = a.ny + 2;
  a.dsx = make_div_magic((unsigned)a.sx);
  a.dsy = make_div_magic((unsigned)a.sy);
  return a;
}

// ahead: nullptr for cell keys, else look-ahead keys on this grid.
static int sort_dispatch(void* particles, void* dst, int64_t num_particles, int64_t num_cells,
                         int32_t precision, int32_t particle_vl, void* d_scratch, size_t need,
                         size_t scratch_bytes, const SortPlan& pl, cudaStream_t s,
                         const cpic_grid* grid = nullptr, const cpic_push_params* prm = nullptr,
                         int steps = 0) {
  if (scratch_bytes < need) return CPIC_ESCRATCH;
  unsigned char* sc = static_cast<unsigned char*>(d_scratch);
  const int n = (int)num_particles, nc = (int)num_cells;
  if (precision == CPIC_FLOAT) {
    const SortAhead<float> a = grid ? make_ahead<float>(grid, prm, steps) : SortAhead<float>{};
    const SortAhead<float>* ap = grid ? &a : nullptr;
    return particle_vl == 32 ? sort_typed<float, 32>(particles, dst, n, nc, pl, sc, ap, s)
                             : sort_typed<float, 16>(particles, dst, n, nc, pl, sc, ap, s);
  }
  const SortAhead<double> a = grid ? make_ahead<double>(grid, prm, steps) : SortAhead<double>{};
  const SortAhead<double>* ap = grid ? &a : nullptr;
  return particle_vl == 32 ? sort_typed<double, 32>(particles, dst, n, nc, pl, sc, ap, s)
                           : sort_typed<double, 16>(particles, dst, n, nc, pl, sc, ap, s);
}

}  // namespace cpic

using namespace cpic;

extern "C" size_t cpic_sort_scratch_bytes(int64_t num_particles, int64_t num_cells, int32_t precision,
                                          int32_t particle_vl) {
  if (num_particles < 0 || num_cells < 1) return 0;
  if (precision != CPIC_FLOAT && precision != CPIC_DOUBLE) return 0;
  if (particle_vl != 16 && particle_vl != 32) return 0;
  return plan_sort(num_particles, num_cells, precision, particle_vl).total;
}

extern "C" int cpic_sort_particles(void* particles, int64_t num_particles, int64_t num_cells,
                                   int32_t precision, int32_t particle_vl, void* d_scratch,
                                   size_t scratch_bytes, cpic_stream_t stream) {
  if (precision != CPIC_FLOAT && precision != CPIC_DOUBLE) return CPIC_EINVAL;
  if (particle_vl != 16 && particle_vl != 32) return CPIC_EINVAL;
  if (num_particles < 0 || num_particles > 0x7fffffffLL - 64) return CPIC_EINVAL;
  if (num_cells < 1 || num_cells > 0x7fffffffLL - 64) return CPIC_EINVAL;
  if (num_particles == 0) return CPIC_OK;
  if (!particles || !d_scratch) return CPIC_EINVAL;
  if (((uintptr_t)particles & 15) || ((uintptr_t)d_scratch & 255)) return CPIC_EINVAL;
  const SortPlan pl = plan_sort(num_particles, num_cells, precision, particle_vl);
  return sort_dispatch(particles, nullptr, num_particles, num_cells, precision, particle_vl, d_scratch,
                       pl.total, scratch_bytes, pl, reinterpret_cast<cudaStream_t>(stream));
}

extern "C" size_t cpic_sort_into_scratch_bytes(int64_t num_particles, int64_t num_cells, int32_t precision,
                                               int32_t particle_vl) {
  if (num_particles < 0 || num_cells < 1) return 0;
  if (precision != CPIC_FLOAT && precision != CPIC_DOUBLE) return 0;
  if (particle_vl != 16 && particle_vl != 32) return 0;
  return plan_sort(num_particles, num_cells, precision, particle_vl).copy_off;
}

extern "C" int cpic_sort_particles_into(const void* particles, void* sorted, int64_t num_particles,
                                        int64_t num_cells, int32_t precision, int32_t particle_vl,
                                        void* d_scratch, size_t scratch_bytes, cpic_stream_t stream) {
  if (precision != CPIC_FLOAT && precision != CPIC_DOUBLE) return CPIC_EINVAL;
  if (particle_vl != 16 && particle_vl != 32) return CPIC_EINVAL;
  if (num_particles < 0 || num_particles > 0x7fffffffLL - 64) return CPIC_EINVAL;
  if (num_cells < 1 || num_cells > 0x7fffffffLL - 64) return CPIC_EINVAL;
  if (num_particles == 0) return CPIC_OK;
  if (!particles || !sorted || !d_scratch) return CPIC_EINVAL;
  {  // the two lists must not overlap
    const uintptr_t bytes = (uintptr_t)cpic_particle_list_bytes(num_particles, precision, particle_vl);
    const uintptr_t a0 = (uintptr_t)particles, b0 = (uintptr_t)sorted;
    if (a0 < b0 + bytes && b0 < a0 + bytes) return CPIC_EINVAL;
  }
  if (((uintptr_t)particles & 15) || ((uintptr_t)sorted & 15) || ((uintptr_t)d_scratch & 255))
    return CPIC_EINVAL;
  const SortPlan pl = plan_sort(num_particles, num_cells, precision, particle_vl);
  return sort_dispatch(const_cast<void*>(particles), sorted, num_particles, num_cells, precision,
                       particle_vl, d_scratch, pl.copy_off, scratch_bytes, pl,
                       reinterpret_cast<cudaStream_t>(stream));
}

extern "C" int cpic_sort_particles_ahead_into(const void* particles, void* sorted, int64_t num_particles,
                                              const cpic_grid* grid, const cpic_push_params* prm,
                                              int32_t steps_ahead, void* d_scratch, size_t scratch_bytes,
                                              cpic_stream_t stream) {
  if (!grid || !prm) return CPIC_EINVAL;
  const int rc = check_grid(grid);
  if (rc) return rc;
  if (prm->precision != CPIC_FLOAT && prm->precision != CPIC_DOUBLE) return CPIC_EINVAL;
  if (prm->particle_vl != 16 && prm->particle_vl != 32) return CPIC_EINVAL;
  if (steps_ahead < 0 || steps_ahead > (1 << 20)) return CPIC_EINVAL;
  if (!(prm->cdt_dx >= 0) || !(prm->cdt_dy >= 0) || !(prm->cdt_dz >= 0)) return CPIC_EINVAL;
  const int64_t num_cells = (int64_t)(grid->nx + 2) * (grid->ny + 2) * (grid->nz + 2);
  if (num_particles < 0 || num_particles > 0x7fffffffLL - 64) return CPIC_EINVAL;
  if (num_particles == 0) return CPIC_OK;
  if (!particles || !sorted || !d_scratch) return CPIC_EINVAL;
  {
    const uintptr_t bytes =
        (uintptr_t)cpic_particle_list_bytes(num_particles, prm->precision, prm->particle_vl);
    const uintptr_t a0 = (uintptr_t)particles, b0 = (uintptr_t)sorted;
    if (a0 < b0 + bytes && b0 < a0 + bytes) return CPIC_EINVAL;
  }
  if (((uintptr_t)particles & 15) || ((uintptr_t)sorted & 15) || ((uintptr_t)d_scratch & 255))
    return CPIC_EINVAL;
  const SortPlan pl = plan_sort(num_particles, num_cells, prm->precision, prm->particle_vl);
  return sort_dispatch(const_cast<void*>(particles), sorted, num_particles, num_cells, prm->precision,
                       prm->particle_vl, d_scratch, pl.copy_off, scratch_bytes, pl,
                       reinterpret_cast<cudaStream_t>(stream), steps_ahead ? grid : nullptr, prm,
                       steps_ahead);
}
