// push.cu -- the exact push variant and the cpic_push / cpic_push_into entry
// points.
//
// The kernel is in push_impl.cuh.  This translation unit is compiled with
// --fmad=false (cabanapic_gb300/build.py) and instantiates it with IEEE
// division and sqrtf: the bit-exact variant, selected with CPIC_PUSH_EXACT.
// push_fast.cu instantiates the default production variant.
#define CPIC_PUSH_NS push_exact
#include "push_impl.cuh"

namespace cpic {
// defined in push_fast.cu
int push_fast_dispatch(void* particles, int n, const void* interp, void* acc, const cpic_grid* g,
                       const cpic_push_params* prm, int* status, cudaStream_t s);
int push_into_fast_dispatch(const void* src, void* dst, int n, const void* interp, void* acc,
                            const cpic_grid* g, const cpic_push_params* prm, int* status, cudaStream_t s);
}  // namespace cpic

namespace {
int check_push_args(int64_t num_particles, const cpic_grid* grid, const cpic_push_params* prm,
                    const int32_t* d_status) {
  using namespace cpic;
  if (!grid || !prm || !d_status) return CPIC_EINVAL;
  int rc = check_grid(grid);
  if (rc) return rc;
  if (num_particles < 0 || num_particles > 0x7fffffffLL - 64) return CPIC_EINVAL;
  if (prm->precision != CPIC_FLOAT && prm->precision != CPIC_DOUBLE) return CPIC_EINVAL;
  if (prm->particle_vl != 16 && prm->particle_vl != 32) return CPIC_EINVAL;
  if (prm->flags & ~(CPIC_PUSH_TRUE_SQRT | CPIC_PUSH_EXACT | CPIC_PUSH_STREAMING | CPIC_PUSH_ACC_F64 |
                     CPIC_PUSH_ACC_LAYOUT_LEFT))
    return CPIC_EINVAL;
  // LayoutLeft with double rows for FP32 particles has no unload entry point
  if ((prm->flags & CPIC_PUSH_ACC_LAYOUT_LEFT) && (prm->flags & CPIC_PUSH_ACC_F64)) return CPIC_EINVAL;
  return CPIC_OK;
}
}  // namespace

extern "C" int cpic_push(void* particles, int64_t num_particles, const void* interpolators,
                         void* accumulators, const cpic_grid* grid, const cpic_push_params* prm,
                         int32_t* d_status, cpic_stream_t stream) {
  using namespace cpic;
  int rc = check_push_args(num_particles, grid, prm, d_status);
  if (rc) return rc;
  if (num_particles == 0) return CPIC_OK;
  if (!particles || !interpolators || !accumulators) return CPIC_EINVAL;
  if (((uintptr_t)accumulators & 15) || ((uintptr_t)particles & 15) ||
      ((uintptr_t)interpolators & 15) || ((uintptr_t)d_status & 3))
    return CPIC_EINVAL;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const int n = (int)num_particles;
  if (prm->flags & CPIC_PUSH_EXACT)
    return push_exact::push_dispatch<false>(particles, n, interpolators, accumulators, grid, prm,
                                            d_status, s);
  return push_fast_dispatch(particles, n, interpolators, accumulators, grid, prm, d_status, s);
}

extern "C" int cpic_push_into(const void* particles, void* out, int64_t num_particles,
                              const void* interpolators, void* accumulators, const cpic_grid* grid,
                              const cpic_push_params* prm, int32_t* d_status, cpic_stream_t stream) {
  using namespace cpic;
  int rc = check_push_args(num_particles, grid, prm, d_status);
  if (rc) return rc;
  if (prm->flags & CPIC_PUSH_STREAMING) return CPIC_EUNSUPPORTED;
  if (num_particles == 0) return CPIC_OK;
  if (!particles || !out || !interpolators || !accumulators) return CPIC_EINVAL;
  {  // the two lists must not overlap
    const uintptr_t bytes = (uintptr_t)cpic_particle_list_bytes(num_particles, prm->precision, prm->particle_vl);
    const uintptr_t a0 = (uintptr_t)particles, b0 = (uintptr_t)out;
    if (a0 < b0 + bytes && b0 < a0 + bytes) return CPIC_EINVAL;
  }
  if (((uintptr_t)accumulators & 15) || ((uintptr_t)particles & 15) || ((uintptr_t)out & 15) ||
      ((uintptr_t)interpolators & 15) || ((uintptr_t)d_status & 3))
    return CPIC_EINVAL;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const int n = (int)num_particles;
  if (prm->flags & CPIC_PUSH_EXACT)
    return push_exact::push_into_dispatch<false>(particles, out, n, interpolators, accumulators, grid, prm,
                                                 d_status, s);
  return push_into_fast_dispatch(particles, out, n, interpolators, accumulators, grid, prm, d_status, s);
}
