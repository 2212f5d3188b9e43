// adjoint_fields.cu -- transposes of the linear per-cell maps of the step, for
// the adjoint (reverse-mode) time step.  No counterpart in the reference.
//
// The field state is periodic: the reference's ghost copies (src/fields.h:
// 11-100), its jf fold (src/fields.h:102-271) and its E update over [1, n+1]
// (src/fields.h:646-664) keep every ghost value equal to the interior value at
// its periodic image.  The forward maps are therefore periodic stencils on the
// interior cells, and their adjoints are the transposed periodic stencils:
//   advance_b   B' = B - Mb E        adjoint: lambda_E -= Mb^T lambda_B
//   advance_e   E' = E - cj J + Me B adjoint: lambda_B += Me^T lambda_E, lambda_J = -cj lambda_E
//   unload      J = U a              adjoint: lambda_a = U^T lambda_J
//   interp      I = P (E, B)         adjoint: lambda_(E,B) += P^T lambda_I
// Every transpose is written as a gather over the interior cells (no
// atomics).  Adjoint arrays use the forward layouts: a field AoSoA holds
// (lambda_E, lambda_B, lambda_J) in the (E, cB, jf) members; ghost cells are
// unused.
#include <cuda_runtime.h>

#include "common.cuh"

namespace cpic {
namespace {

constexpr int kAdjThreads = 256;
constexpr int kAdjRow = CPIC_ADJ_INTERP_ROW;  // values per row of a row-layout interpolator adjoint

struct Periodic {
  GridDev g;
  __device__ int xp(int x) const { return x == g.nx ? 1 : x + 1; }
  __device__ int xm(int x) const { return x == 1 ? g.nx : x - 1; }
  __device__ int yp(int y) const { return y == g.ny ? 1 : y + 1; }
  __device__ int ym(int y) const { return y == 1 ? g.ny : y - 1; }
  __device__ int zp(int z) const { return z == g.nz ? 1 : z + 1; }
  __device__ int zm(int z) const { return z == 1 ? g.nz : z - 1; }
};

// This thread's interior cell (aligned 32-cell blocks of the linear index).
__device__ __forceinline__ bool interior_cell(int begin, int end, const GridDev& g, int& j, int& x, int& y,
                                              int& z) {
  j = lane_cell0<1, kAdjThreads>(begin);
  return cell_in_box(j, end, g, g.nx, g.ny, g.nz, x, y, z);
}

template <class R>
__device__ __forceinline__ R& fm(R* F, int c, int m) { return F[cell_at<9>(c, m)]; }

// lambda_E -= Mb^T lambda_B, with Mb the forward-difference curl of advance_b
// (src/fields.h:707-709) and coefficients (px, py, pz).
template <class R>
__global__ void __launch_bounds__(kAdjThreads)
adj_advance_b_kernel(R* __restrict__ L, const GridDev g, R px, R py, R pz, int begin, int end) {
  int j, x, y, z;
  if (!interior_cell(begin, end, g, j, x, y, z)) return;
  const Periodic P{g};
  const int jxm = g.vox(P.xm(x), y, z), jym = g.vox(x, P.ym(y), z), jzm = g.vox(x, y, P.zm(z));
  const R bx = fm(L, j, CPIC_F_CBX), by = fm(L, j, CPIC_F_CBY), bz = fm(L, j, CPIC_F_CBZ);
  const R tex = pz * (fm(L, jzm, CPIC_F_CBY) - by) - py * (fm(L, jym, CPIC_F_CBZ) - bz);
  const R tey = px * (fm(L, jxm, CPIC_F_CBZ) - bz) - pz * (fm(L, jzm, CPIC_F_CBX) - bx);
  const R tez = py * (fm(L, jym, CPIC_F_CBX) - bx) - px * (fm(L, jxm, CPIC_F_CBY) - by);
  fm(L, j, CPIC_F_EX) -= tex;
  fm(L, j, CPIC_F_EY) -= tey;
  fm(L, j, CPIC_F_EZ) -= tez;
}

// lambda_B += Me^T lambda_E and lambda_J = -cj lambda_E, with Me the
// backward-difference curl of advance_e (src/fields.h:655-657).
template <class R>
__global__ void __launch_bounds__(kAdjThreads)
adj_advance_e_kernel(R* __restrict__ L, const GridDev g, R px, R py, R pz, R cj, int begin, int end) {
  int j, x, y, z;
  if (!interior_cell(begin, end, g, j, x, y, z)) return;
  const Periodic P{g};
  const int jxp = g.vox(P.xp(x), y, z), jyp = g.vox(x, P.yp(y), z), jzp = g.vox(x, y, P.zp(z));
  const R ex = fm(L, j, CPIC_F_EX), ey = fm(L, j, CPIC_F_EY), ez = fm(L, j, CPIC_F_EZ);
  fm(L, j, CPIC_F_CBX) += pz * (ey - fm(L, jzp, CPIC_F_EY)) - py * (ez - fm(L, jyp, CPIC_F_EZ));
  fm(L, j, CPIC_F_CBY) += px * (ez - fm(L, jxp, CPIC_F_EZ)) - pz * (ex - fm(L, jzp, CPIC_F_EX));
  fm(L, j, CPIC_F_CBZ) += py * (ex - fm(L, jyp, CPIC_F_EX)) - px * (ey - fm(L, jxp, CPIC_F_EY));
  fm(L, j, CPIC_F_JFX) = -cj * ex;
  fm(L, j, CPIC_F_JFY) = -cj * ey;
  fm(L, j, CPIC_F_JFZ) = -cj * ez;
}

// lambda_a = U^T lambda_J, U the periodic unload (src/accumulator.cpp:71-110
// with the jf fold); writes the 12 adjoint accumulators of every interior cell.
__device__ __forceinline__ void st4(float* p, float a, float b, float c, float d) {
  *reinterpret_cast<float4*>(p) = make_float4(a, b, c, d);
}
__device__ __forceinline__ void st4(double* p, double a, double b, double c, double d) {
  reinterpret_cast<double2*>(p)[0] = make_double2(a, b);
  reinterpret_cast<double2*>(p)[1] = make_double2(c, d);
}

template <class R>
__global__ void __launch_bounds__(kAdjThreads)
adj_unload_kernel(const R* __restrict__ L, R* __restrict__ A, const GridDev g, R cx, R cy, R cz, int begin, int end) {
  int c, x, y, z;
  if (!interior_cell(begin, end, g, c, x, y, z)) return;
  const Periodic P{g};
  const int xp = P.xp(x), yp = P.yp(y), zp = P.zp(z);
  auto lj = [&](int cc, int m) { return L[cell_at<9>(cc, m)]; };
  // the cell's 48-byte row (16-byte aligned) in three 4-value stores
  R* a = A + (size_t)c * 12;
  st4(a, cx * lj(c, CPIC_F_JFX), cx * lj(g.vox(x, yp, z), CPIC_F_JFX), cx * lj(g.vox(x, y, zp), CPIC_F_JFX),
      cx * lj(g.vox(x, yp, zp), CPIC_F_JFX));
  st4(a + 4, cy * lj(c, CPIC_F_JFY), cy * lj(g.vox(x, y, zp), CPIC_F_JFY), cy * lj(g.vox(xp, y, z), CPIC_F_JFY),
      cy * lj(g.vox(xp, y, zp), CPIC_F_JFY));
  st4(a + 8, cz * lj(c, CPIC_F_JFZ), cz * lj(g.vox(xp, y, z), CPIC_F_JFZ), cz * lj(g.vox(x, yp, z), CPIC_F_JFZ),
      cz * lj(g.vox(xp, yp, z), CPIC_F_JFZ));
}

// lambda_(E, B) += P^T lambda_I, P the interpolator load
// (src/interpolator.cpp:80-131): each field value feeds the coefficients of up
// to four cells (E) or two cells (B); gathered per field cell.
// Four (or two) consecutive coefficients of one cell.  In the row layout a
// bilinear block (members 4k..4k+3) is 16-byte aligned and a cB pair 8-byte
// aligned, so each is one vector load (two for double).
template <class R>
struct Q4 {
  R a, b, c, d;
};
__device__ __forceinline__ Q4<float> ld_q4(const float* p) {
  const float4 v = *reinterpret_cast<const float4*>(p);
  return {v.x, v.y, v.z, v.w};
}
__device__ __forceinline__ Q4<double> ld_q4(const double* p) {
  const double2 v0 = *reinterpret_cast<const double2*>(p), v1 = *reinterpret_cast<const double2*>(p + 2);
  return {v0.x, v0.y, v1.x, v1.y};
}
__device__ __forceinline__ float2 ld_q2(const float* p) { return *reinterpret_cast<const float2*>(p); }
__device__ __forceinline__ double2 ld_q2(const double* p) { return *reinterpret_cast<const double2*>(p); }

template <class R, bool ROWS = false>
__global__ void __launch_bounds__(kAdjThreads)
adj_interp_kernel(const R* __restrict__ LI, R* __restrict__ L, const GridDev g, int begin, int end) {
  int j, x, y, z;
  if (!interior_cell(begin, end, g, j, x, y, z)) return;
  const Periodic P{g};
  const int xm = P.xm(x), ym = P.ym(y), zm = P.zm(z);
  // ROWS: the interpolator adjoint in cell-major rows of kAdjRow values
  auto blk = [&](int c, int m) -> Q4<R> {
    if constexpr (ROWS) return ld_q4(LI + (size_t)c * kAdjRow + m);
    else return {LI[cell_at<18>(c, m)], LI[cell_at<18>(c, m + 1)], LI[cell_at<18>(c, m + 2)],
                 LI[cell_at<18>(c, m + 3)]};
  };
  auto pair = [&](int c, int m, R& v0, R& v1) {
    if constexpr (ROWS) {
      const auto v = ld_q2(LI + (size_t)c * kAdjRow + m);
      v0 = v.x; v1 = v.y;
    } else {
      v0 = LI[cell_at<18>(c, m)]; v1 = LI[cell_at<18>(c, m + 1)];
    }
  };
  const R q = 0.25, h = 0.5;
  // the four weights of a bilinear coefficient block (value, d/da, d/db, d2/dadb)
  // for corners w0 (own), w1 (+a), w2 (+b), w3 (+a+b)
  auto w0 = [&](int c, int m) { const Q4<R> v = blk(c, m); return q * (v.a - v.b - v.c + v.d); };
  auto w1 = [&](int c, int m) { const Q4<R> v = blk(c, m); return q * (v.a + v.b - v.c - v.d); };
  auto w2 = [&](int c, int m) { const Q4<R> v = blk(c, m); return q * (v.a - v.b + v.c - v.d); };
  auto w3 = [&](int c, int m) { const Q4<R> v = blk(c, m); return q * (v.a + v.b + v.c + v.d); };
  // ex: corners (i, i+y, i+z, i+y+z)
  fm(L, j, CPIC_F_EX) += w0(j, CPIC_I_EX) + w1(g.vox(x, ym, z), CPIC_I_EX) +
                         w2(g.vox(x, y, zm), CPIC_I_EX) + w3(g.vox(x, ym, zm), CPIC_I_EX);
  // ey: corners (i, i+z, i+x, i+x+z)
  fm(L, j, CPIC_F_EY) += w0(j, CPIC_I_EY) + w1(g.vox(x, y, zm), CPIC_I_EY) +
                         w2(g.vox(xm, y, z), CPIC_I_EY) + w3(g.vox(xm, y, zm), CPIC_I_EY);
  // ez: corners (i, i+x, i+y, i+x+y)
  fm(L, j, CPIC_F_EZ) += w0(j, CPIC_I_EZ) + w1(g.vox(xm, y, z), CPIC_I_EZ) +
                         w2(g.vox(x, ym, z), CPIC_I_EZ) + w3(g.vox(xm, ym, z), CPIC_I_EZ);
  // cbx: (i, i+x); cby: (i, i+y); cbz: (i, i+z)
  R a0, a1, b0, b1;
  pair(j, CPIC_I_CBX, a0, a1);
  pair(g.vox(xm, y, z), CPIC_I_CBX, b0, b1);
  fm(L, j, CPIC_F_CBX) += h * (a0 - a1) + h * (b0 + b1);
  pair(j, CPIC_I_CBY, a0, a1);
  pair(g.vox(x, ym, z), CPIC_I_CBY, b0, b1);
  fm(L, j, CPIC_F_CBY) += h * (a0 - a1) + h * (b0 + b1);
  pair(j, CPIC_I_CBZ, a0, a1);
  pair(g.vox(x, y, zm), CPIC_I_CBZ, b0, b1);
  fm(L, j, CPIC_F_CBZ) += h * (a0 - a1) + h * (b0 + b1);
}

static_assert(CPIC_I_EY == CPIC_I_EX + 4 && CPIC_I_EZ == CPIC_I_EX + 8 && CPIC_I_EX == 0,
              "bilinear blocks at members 0, 4, 8");
static_assert(CPIC_I_DCBXDX == CPIC_I_CBX + 1 && CPIC_I_DCBYDY == CPIC_I_CBY + 1 &&
                  CPIC_I_DCBZDZ == CPIC_I_CBZ + 1 && CPIC_I_CBX % 2 == 0 && CPIC_I_CBY % 2 == 0 &&
                  CPIC_I_CBZ % 2 == 0,
              "cB pairs at even members");
static_assert(CPIC_ADJ_INTERP_ROW % 4 == 0, "rows of a multiple of 16 bytes");

inline CellRange interior_range(const GridDev& g) { return cell_range<1, kAdjThreads>(g, g.nx, g.ny, g.nz); }

}  // namespace
}  // namespace cpic

using namespace cpic;

#define ADJ_PREAMBLE()                                                    \
  int rc = check_grid(grid);                                              \
  if (rc) return rc;                                                      \
  if (precision != CPIC_FLOAT && precision != CPIC_DOUBLE) return CPIC_EINVAL; \
  const GridDev g = make_grid(grid);                                      \
  const CellRange r = interior_range(g);                                  \
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream)

extern "C" int cpic_adjoint_advance_b(void* d_lambda_fields, double px, double py, double pz,
                                      const cpic_grid* grid, int32_t precision, cpic_stream_t stream) {
  ADJ_PREAMBLE();
  if (!d_lambda_fields) return CPIC_EINVAL;
  if (precision == CPIC_FLOAT)
    adj_advance_b_kernel<float><<<r.blocks, kAdjThreads, 0, s>>>(static_cast<float*>(d_lambda_fields), g,
                                                                   (float)px, (float)py, (float)pz, r.begin, r.end);
  else
    adj_advance_b_kernel<double><<<r.blocks, kAdjThreads, 0, s>>>(static_cast<double*>(d_lambda_fields), g,
                                                                    px, py, pz, r.begin, r.end);
  return launch_status();
}

extern "C" int cpic_adjoint_advance_e(void* d_lambda_fields, double px, double py, double pz,
                                      const cpic_grid* grid, double dt_eps0, int32_t precision,
                                      cpic_stream_t stream) {
  ADJ_PREAMBLE();
  if (!d_lambda_fields) return CPIC_EINVAL;
  if (precision == CPIC_FLOAT)
    adj_advance_e_kernel<float><<<r.blocks, kAdjThreads, 0, s>>>(static_cast<float*>(d_lambda_fields), g,
                                                                   (float)px, (float)py, (float)pz,
                                                                   (float)dt_eps0, r.begin, r.end);
  else
    adj_advance_e_kernel<double><<<r.blocks, kAdjThreads, 0, s>>>(static_cast<double*>(d_lambda_fields), g,
                                                                    px, py, pz, dt_eps0, r.begin, r.end);
  return launch_status();
}

extern "C" int cpic_adjoint_unload_accumulator(const void* d_lambda_fields, void* d_lambda_acc,
                                               const cpic_grid* grid, double dx, double dy, double dz,
                                               double dt, int32_t precision, cpic_stream_t stream) {
  ADJ_PREAMBLE();
  if (!d_lambda_fields || !d_lambda_acc) return CPIC_EINVAL;
  if ((uintptr_t)d_lambda_acc & 15) return CPIC_EINVAL;  // rows written with vector stores
  if (precision == CPIC_FLOAT) {
    const float rdx = (float)dx, rdy = (float)dy, rdz = (float)dz, rdt = (float)dt;
    adj_unload_kernel<float><<<r.blocks, kAdjThreads, 0, s>>>(
        static_cast<const float*>(d_lambda_fields), static_cast<float*>(d_lambda_acc), g,
        (float)(0.25 / (double)(float)(rdy * rdz * rdt)), (float)(0.25 / (double)(float)(rdz * rdx * rdt)),
        (float)(0.25 / (double)(float)(rdx * rdy * rdt)), r.begin, r.end);
  } else {
    adj_unload_kernel<double><<<r.blocks, kAdjThreads, 0, s>>>(
        static_cast<const double*>(d_lambda_fields), static_cast<double*>(d_lambda_acc), g,
        0.25 / (dy * dz * dt), 0.25 / (dz * dx * dt), 0.25 / (dx * dy * dt), r.begin, r.end);
  }
  return launch_status();
}

extern "C" int cpic_adjoint_load_interpolator_rows(const void* d_lambda_interp_rows, void* d_lambda_fields,
                                                   const cpic_grid* grid, int32_t precision,
                                                   cpic_stream_t stream) {
  ADJ_PREAMBLE();
  if (!d_lambda_interp_rows || !d_lambda_fields) return CPIC_EINVAL;
  if ((uintptr_t)d_lambda_interp_rows & 15) return CPIC_EINVAL;  // rows are read with vector loads
  if (precision == CPIC_FLOAT)
    adj_interp_kernel<float, true><<<r.blocks, kAdjThreads, 0, s>>>(
        static_cast<const float*>(d_lambda_interp_rows), static_cast<float*>(d_lambda_fields), g, r.begin, r.end);
  else
    adj_interp_kernel<double, true><<<r.blocks, kAdjThreads, 0, s>>>(
        static_cast<const double*>(d_lambda_interp_rows), static_cast<double*>(d_lambda_fields), g, r.begin, r.end);
  return launch_status();
}

extern "C" int cpic_adjoint_load_interpolator(const void* d_lambda_interp, void* d_lambda_fields,
                                              const cpic_grid* grid, int32_t precision,
                                              cpic_stream_t stream) {
  ADJ_PREAMBLE();
  if (!d_lambda_interp || !d_lambda_fields) return CPIC_EINVAL;
  if (precision == CPIC_FLOAT)
    adj_interp_kernel<float><<<r.blocks, kAdjThreads, 0, s>>>(static_cast<const float*>(d_lambda_interp),
                                                                static_cast<float*>(d_lambda_fields), g, r.begin, r.end);
  else
    adj_interp_kernel<double><<<r.blocks, kAdjThreads, 0, s>>>(static_cast<const double*>(d_lambda_interp),
                                                                 static_cast<double*>(d_lambda_fields), g, r.begin, r.end);
  return launch_status();
}
