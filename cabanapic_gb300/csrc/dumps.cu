// dumps.cu -- the values the reference's text dumps print, computed on the
// device so that only 2 reals per particle (or per x cell) cross to the host:
//   dump_particles (src/helpers.h:31-61): x = xmin + (ix - 1 + (px + 1) 0.5) dx
//     in double, stored as real_t, and ux, for every particle;
//   Field_Solver::dump_fields (src/fields.h:318-350): x = xmin + (i - 0.5) dx
//     and ex of voxel (i, 1, 1), for i = 1..nx.
// The host formats them ("%e  %e " per particle, "%e %e\n" per cell) after an
// asynchronous copy, so a dump does not stall the time loop.
#include <cuda_runtime.h>

#include "common.cuh"

namespace cpic {
namespace {

template <class R, int VL>
__global__ void __launch_bounds__(256)
particle_dump_kernel(const unsigned char* __restrict__ part, int n, int sx, R xmin, R dx,
                     R* __restrict__ out) {
  using L = PLayout<R, VL>;
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const R px = *reinterpret_cast<const R*>(part + L::off(p, 0));
  const R ux = *reinterpret_cast<const R*>(part + L::off(p, 3));
  const int cell = *reinterpret_cast<const int*>(part + L::cell_off(p));
  const int ix = cell - sx * (cell / sx);  // RANK_TO_INDEX (src/types.h:184-193)
  const double x = (double)xmin + ((double)(ix - 1) + ((double)px + 1.0) * 0.5) * (double)dx;
  out[2 * p] = (R)x;
  out[2 * p + 1] = ux;
}

template <class R>
__global__ void __launch_bounds__(256)
field_dump_kernel(const R* __restrict__ fields, GridDev g, R xmin, R dx, R* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;  // 1..nx
  if (i > g.nx) return;
  const double x = (double)xmin + ((double)i - 0.5) * (double)dx;
  out[2 * (i - 1)] = (R)x;
  out[2 * (i - 1) + 1] = fields[cell_at<9>(g.vox(i, 1, 1), CPIC_F_EX)];
}

}  // namespace
}  // namespace cpic

extern "C" int cpic_particle_dump_values(const void* particles, int64_t num_particles, int32_t particle_vl,
                                         const cpic_grid* grid, int32_t precision, double xmin, double dx,
                                         void* d_out, cpic_stream_t stream) {
  using namespace cpic;
  int rc = check_grid(grid);
  if (rc) return rc;
  if (precision != CPIC_FLOAT && precision != CPIC_DOUBLE) return CPIC_EINVAL;
  if (particle_vl != 16 && particle_vl != 32) return CPIC_EINVAL;
  if (num_particles < 0 || num_particles > 0x7fffffffLL - 64) return CPIC_EINVAL;
  if (num_particles == 0) return CPIC_OK;
  if (!particles || !d_out) return CPIC_EINVAL;
  const GridDev g = make_grid(grid);
  const int n = (int)num_particles;
  const unsigned blocks = (unsigned)((n + 255) / 256);
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const auto* part = static_cast<const unsigned char*>(particles);
  if (precision == CPIC_FLOAT) {
    float* o = static_cast<float*>(d_out);
    if (particle_vl == 32) particle_dump_kernel<float, 32><<<blocks, 256, 0, s>>>(part, n, g.sx, (float)xmin, (float)dx, o);
    else particle_dump_kernel<float, 16><<<blocks, 256, 0, s>>>(part, n, g.sx, (float)xmin, (float)dx, o);
  } else {
    double* o = static_cast<double*>(d_out);
    if (particle_vl == 32) particle_dump_kernel<double, 32><<<blocks, 256, 0, s>>>(part, n, g.sx, xmin, dx, o);
    else particle_dump_kernel<double, 16><<<blocks, 256, 0, s>>>(part, n, g.sx, xmin, dx, o);
  }
  return launch_status();
}

extern "C" int cpic_field_dump_values(const void* fields, const cpic_grid* grid, int32_t precision,
                                      double xmin, double dx, void* d_out, cpic_stream_t stream) {
  using namespace cpic;
  int rc = check_grid(grid);
  if (rc) return rc;
  if (precision != CPIC_FLOAT && precision != CPIC_DOUBLE) return CPIC_EINVAL;
  if (!fields || !d_out) return CPIC_EINVAL;
  const GridDev g = make_grid(grid);
  const unsigned blocks = (unsigned)((g.nx + 255) / 256);
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  if (precision == CPIC_FLOAT)
    field_dump_kernel<float><<<blocks, 256, 0, s>>>(static_cast<const float*>(fields), g, (float)xmin,
                                                    (float)dx, static_cast<float*>(d_out));
  else
    field_dump_kernel<double><<<blocks, 256, 0, s>>>(static_cast<const double*>(fields), g, xmin, dx,
                                                     static_cast<double*>(d_out));
  return launch_status();
}
