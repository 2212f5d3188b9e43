// uncenter.cu -- uncenter_particles (reference src/uncenter_p.h:4-105): the
// optional back half-step of momentum at t = 0 (example/example.cpp:204-213):
// a Boris rotation with -qdt_2mc/2, then the half E kick, as the reference
// writes them.  Compiled with --fmad=false: bit-identical to a CPU build of
// the reference without FMA contraction.
#include <cuda_runtime.h>

#include "common.cuh"

namespace cpic {
namespace {

template <class R, int VL>
__global__ void __launch_bounds__(256)
uncenter_kernel(unsigned char* __restrict__ part, int n, const R* __restrict__ interp, R qdt_2mc,
                int num_cells, int* __restrict__ status) {
  using L = PLayout<R, VL>;
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const R qdt_4mc = (R)(-0.5 * (double)qdt_2mc);
  const R one = 1., one_third = 1. / 3., two_fifteenths = 2. / 15.;
  auto mem = [&](int m) -> R& { return *reinterpret_cast<R*>(part + L::off(p, m)); };
  const int ii = *reinterpret_cast<const int*>(part + L::cell_off(p));
  if ((unsigned)ii >= (unsigned)num_cells) {
    atomicOr(status, CPIC_STATUS_CELL_RANGE);
    return;
  }
  const R dx = mem(0), dy = mem(1), dz = mem(2);
  const R* f = interp + ((size_t)(ii >> 5) * (18 * kCellBlock) + (ii & 31));
  auto c = [&](int m) { return __ldg(f + m * 32); };
  const R hax = qdt_2mc * ((c(0) + dy * c(1)) + dz * (c(2) + dy * c(3)));
  const R hay = qdt_2mc * ((c(4) + dz * c(5)) + dx * (c(6) + dz * c(7)));
  const R haz = qdt_2mc * ((c(8) + dx * c(9)) + dy * (c(10) + dx * c(11)));
  const R cbx = c(12) + dx * c(13), cby = c(14) + dy * c(15), cbz = c(16) + dz * c(17);
  R ux = mem(3), uy = mem(4), uz = mem(5);
  // v0 = qdt_4mc / (real_t)sqrt(...) (uncenter_p.h:72)
  R s;
  if constexpr (sizeof(R) == 8) s = sqrt(one + (ux * ux + (uy * uy + uz * uz)));
  else s = sqrtf(one + (ux * ux + (uy * uy + uz * uz)));
  const R v0 = qdt_4mc / s;
  const R v1 = cbx * cbx + (cby * cby + cbz * cbz);
  const R v2 = (v0 * v0) * v1;
  const R v3 = v0 * (one + v2 * (one_third + v2 * two_fifteenths));
  R v4 = v3 / (one + v1 * (v3 * v3));
  v4 += v4;
  const R t0 = ux + v3 * (uy * cbz - uz * cby);
  const R t1 = uy + v3 * (uz * cbx - ux * cbz);
  const R t2 = uz + v3 * (ux * cby - uy * cbx);
  ux += v4 * (t1 * cbz - t2 * cby);
  uy += v4 * (t2 * cbx - t0 * cbz);
  uz += v4 * (t0 * cby - t1 * cbx);
  ux += hax; uy += hay; uz += haz;
  mem(3) = ux; mem(4) = uy; mem(5) = uz;
}

template <class R>
int typed(void* part, int n, const void* interp, double qdt_2mc, int vl, int nc, int* st, cudaStream_t s) {
  const unsigned blocks = (unsigned)(((int64_t)n + 255) / 256);
  if (vl == 32)
    uncenter_kernel<R, 32><<<blocks, 256, 0, s>>>(static_cast<unsigned char*>(part), n,
                                                   static_cast<const R*>(interp), (R)qdt_2mc, nc, st);
  else
    uncenter_kernel<R, 16><<<blocks, 256, 0, s>>>(static_cast<unsigned char*>(part), n,
                                                   static_cast<const R*>(interp), (R)qdt_2mc, nc, st);
  return launch_status();
}

}  // namespace
}  // namespace cpic

extern "C" int cpic_uncenter_particles(void* particles, int64_t num_particles, const void* interpolators,
                                       double qdt_2mc, const cpic_grid* grid, int32_t precision,
                                       int32_t particle_vl, int32_t* d_status, cpic_stream_t stream) {
  using namespace cpic;
  int rc = check_grid(grid);
  if (rc) return rc;
  if (precision != CPIC_FLOAT && precision != CPIC_DOUBLE) return CPIC_EINVAL;
  if (particle_vl != 16 && particle_vl != 32) return CPIC_EINVAL;
  if (num_particles < 0 || num_particles > 0x7fffffffLL - 64) return CPIC_EINVAL;
  if (num_particles == 0) return CPIC_OK;
  if (!particles || !interpolators || !d_status) return CPIC_EINVAL;
  const GridDev g = make_grid(grid);
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const int n = (int)num_particles;
  return precision == CPIC_FLOAT
             ? typed<float>(particles, n, interpolators, qdt_2mc, particle_vl, g.num_cells, d_status, s)
             : typed<double>(particles, n, interpolators, qdt_2mc, particle_vl, g.num_cells, d_status, s);
}
