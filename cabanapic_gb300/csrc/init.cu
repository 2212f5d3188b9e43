// init.cu -- seeded particle loading on the device for the uniform thermal
// plasma: ppc electrons per interior cell, cells in VOXEL order (x fastest),
// uniform in-cell offsets in [-1, 1) and Maxwellian momenta of width u_th per
// component, every particle with the same weight.
//
// The random numbers come from Philox4x32-10 (Salmon, Moraes, Dror, Shaw,
// "Parallel random numbers: as easy as 1, 2, 3", SC'11), a counter-based
// generator: particle p draws from counters (p, 0) and (p, 1) under the key
// (seed), so every particle's values depend only on (seed, p) -- no state, no
// ordering between threads, and the same values on any device or on the host
// (cabanapic_gb300/decks.py restates the generator with numpy).
//   x, y, z = 2 u - 1 with u from one 32-bit output (24 bits for FP32);
//   ux, uy  = u_th sqrt(-2 ln a) (cos, sin)(2 pi b)   (Box-Muller)
//   uz      = u_th sqrt(-2 ln c) cos(2 pi d)
// the normals computed in double and rounded once to real_t.
#include <cuda_runtime.h>

#include "common.cuh"

namespace cpic {
namespace {

struct U4 {
  unsigned x, y, z, w;
};

// Philox4x32 with 10 rounds: per round, two 32x32->64 multiplies of counter
// words 0 and 2, the high halves mixed with words 1 and 3 and the key; the
// key is bumped by the Weyl constants between rounds.
__device__ __forceinline__ U4 philox4x32_10(U4 c, unsigned k0, unsigned k1) {
  constexpr unsigned kM0 = 0xD2511F53u, kM1 = 0xCD9E8D57u;
  constexpr unsigned kW0 = 0x9E3779B9u, kW1 = 0xBB67AE85u;
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const unsigned lo0 = kM0 * c.x, hi0 = __umulhi(kM0, c.x);
    const unsigned lo1 = kM1 * c.z, hi1 = __umulhi(kM1, c.z);
    c = U4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
    k0 += kW0;
    k1 += kW1;
  }
  return c;
}

template <class R>
__device__ __forceinline__ R offset_of(unsigned r);

template <>
__device__ __forceinline__ float offset_of<float>(unsigned r) {
  return (float)(r >> 8) * 0x1p-23f - 1.0f;  // 2 (r >> 8) 2^-24 - 1, exact
}

template <>
__device__ __forceinline__ double offset_of<double>(unsigned r) {
  return (double)r * 0x1p-31 - 1.0;  // 2 r 2^-32 - 1, exact
}

template <class R, int VL>
__global__ void __launch_bounds__(256)
thermal_init_kernel(unsigned char* __restrict__ part, int64_t n, int ppc, int nx, int ny, int sx, int sy,
                    double uth, R weight, unsigned k0, unsigned k1) {
  using L = PLayout<R, VL>;
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const int64_t k = p / ppc;  // interior cell, x fastest
  const int ix = (int)(k % nx), iy = (int)((k / nx) % ny), iz = (int)(k / ((int64_t)nx * ny));
  const int cell = (ix + 1) + sx * ((iy + 1) + sy * (iz + 1));
  const unsigned plo = (unsigned)p, phi = (unsigned)((uint64_t)p >> 32);
  const U4 a = philox4x32_10(U4{plo, phi, 0u, 0u}, k0, k1);
  const U4 b = philox4x32_10(U4{plo, phi, 1u, 0u}, k0, k1);
  const double r1 = sqrt(-2.0 * log(((double)a.w + 1.0) * 0x1p-32));
  const double r2 = sqrt(-2.0 * log(((double)b.y + 1.0) * 0x1p-32));
  double s1, c1;
  sincospi(2.0 * ((double)b.x * 0x1p-32), &s1, &c1);
  const double c2 = cospi(2.0 * ((double)b.z * 0x1p-32));
  *reinterpret_cast<R*>(part + L::off(p, 0)) = offset_of<R>(a.x);
  *reinterpret_cast<R*>(part + L::off(p, 1)) = offset_of<R>(a.y);
  *reinterpret_cast<R*>(part + L::off(p, 2)) = offset_of<R>(a.z);
  *reinterpret_cast<R*>(part + L::off(p, 3)) = (R)(uth * (r1 * c1));
  *reinterpret_cast<R*>(part + L::off(p, 4)) = (R)(uth * (r1 * s1));
  *reinterpret_cast<R*>(part + L::off(p, 5)) = (R)(uth * (r2 * c2));
  *reinterpret_cast<R*>(part + L::off(p, 6)) = weight;
  *reinterpret_cast<int*>(part + L::cell_off(p)) = cell;
}

template <class R, int VL>
int launch_thermal(void* particles, int64_t n, int ppc, const cpic_grid* g, double uth, double weight,
                   uint64_t seed, cudaStream_t s) {
  const unsigned blocks = (unsigned)((n + 255) / 256);
  thermal_init_kernel<R, VL><<<blocks, 256, 0, s>>>(
      static_cast<unsigned char*>(particles), n, ppc, (int)g->nx, (int)g->ny, (int)g->nx + 2, (int)g->ny + 2,
      uth, (R)weight, (unsigned)seed, (unsigned)(seed >> 32));
  return launch_status();
}

}  // namespace
}  // namespace cpic

using namespace cpic;

extern "C" int cpic_thermal_particles(void* particles, int64_t num_particles, int32_t ppc,
                                      const cpic_grid* grid, double uth, double weight, uint64_t seed,
                                      int32_t precision, int32_t particle_vl, cpic_stream_t stream) {
  const int rc = check_grid(grid);
  if (rc) return rc;
  if (precision != CPIC_FLOAT && precision != CPIC_DOUBLE) return CPIC_EINVAL;
  if (particle_vl != 16 && particle_vl != 32) return CPIC_EINVAL;
  if (ppc < 1 || num_particles < 0 || num_particles > 0x7fffffffLL - 64) return CPIC_EINVAL;
  if (num_particles > (int64_t)ppc * grid->nx * grid->ny * grid->nz) return CPIC_EINVAL;
  if (!(uth >= 0.0)) return CPIC_EINVAL;
  if (num_particles == 0) return CPIC_OK;
  if (!particles || ((uintptr_t)particles & 15)) return CPIC_EINVAL;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  if (precision == CPIC_FLOAT)
    return particle_vl == 32 ? launch_thermal<float, 32>(particles, num_particles, ppc, grid, uth, weight, seed, s)
                             : launch_thermal<float, 16>(particles, num_particles, ppc, grid, uth, weight, seed, s);
  return particle_vl == 32 ? launch_thermal<double, 32>(particles, num_particles, ppc, grid, uth, weight, seed, s)
                           : launch_thermal<double, 16>(particles, num_particles, ppc, grid, uth, weight, seed, s);
}
