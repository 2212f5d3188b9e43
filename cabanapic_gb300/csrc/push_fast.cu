// push_fast.cu -- the production push variant (the cpic_push default).
//
// The kernel is in push_impl.cuh.  This translation unit is compiled with
// fused multiply-adds (--fmad=true, cabanapic_gb300/build.py) and instantiates
// it with the hardware reciprocal and reciprocal square root for the FP32
// gamma and Boris divisions.  Per-particle results agree with the exact
// variant (push.cu) to ~1e-6 relative; the tests hold them to 1e-5.
#define CPIC_PUSH_NS push_fast
#include "push_impl.cuh"

namespace cpic {

int push_fast_dispatch(void* particles, int n, const void* interp, void* acc, const cpic_grid* g,
                       const cpic_push_params* prm, int* status, cudaStream_t s) {
  return push_fast::push_dispatch<true>(particles, n, interp, acc, g, prm, status, s);
}

int push_into_fast_dispatch(const void* src, void* dst, int n, const void* interp, void* acc,
                            const cpic_grid* g, const cpic_push_params* prm, int* status, cudaStream_t s) {
  return push_fast::push_into_dispatch<true>(src, dst, n, interp, acc, g, prm, status, s);
}

}  // namespace cpic
