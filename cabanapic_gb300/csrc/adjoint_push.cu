// adjoint_push.cu -- reverse-mode (vector-Jacobian product) of push() for the
// adjoint time step.  No counterpart in the reference.
//
// Forward map of one particle (src/push.h:66-295, src/move_p.h:93-371):
//   (offsets x, momentum u, interpolator coefficients f[18] of its cell)
//     -> (new offsets x', new momentum u', 12 current deposits per streak).
// Given the adjoints of the outputs -- lambda_x', lambda_u' (the particle's
// adjoint after the step) and lambda_a (the adjoint of the accumulator array,
// read at the cells the particle deposits into: the transpose of the deposit
// is a gather from the adjoint currents) -- the kernel recomputes the forward
// push from the step's starting state and returns lambda_x, lambda_u (the
// adjoint before the step, written in place) and adds lambda_f to the
// adjoint interpolator array (the transpose of the gather: reduced over the
// warp's largest group of lanes sharing a cell, then atomics).
//
// Cell indices are piecewise constant: the streak split (which face is hit
// first, how many streaks) is taken from the forward recompute, and the
// derivative flows through the streak lengths and midpoints.  The particle
// weight is not differentiated.
//
// This unit is built with fused multiply-adds and the fast FP32 divide and
// square root (cabanapic_gb300/build.py): its results are held to finite
// differences within a tolerance, not to another implementation bit for bit.
#include <cuda_runtime.h>

#include "common.cuh"

namespace cpic {
namespace {

constexpr int kAdjThreads = 128;
constexpr int kMaxAdjStreaks = 8;  // a Courant-limited move needs at most 4

template <class R>
struct AdjArgs {
  R qdt_2mc, cdt_dx, cdt_dy, cdt_dz, qsp;
  GridDev g;
};

template <class R>
struct V3 {
  R x, y, z;
};
template <class R>
__device__ __forceinline__ V3<R> cross(V3<R> a, V3<R> b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class R>
__device__ __forceinline__ R dot(V3<R> a, V3<R> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

template <class R, bool LITERAL>
__device__ __forceinline__ R root(R a) {
  if constexpr (sizeof(R) == 8 && LITERAL) return (R)sqrtf((float)a);
  else if constexpr (sizeof(R) == 8) return sqrt(a);
  else return sqrtf(a);
}

// Adjoint of the 12 deposits of one streak: currents of charge q, streak s,
// midpoint m (src/push.h:218-254, src/move_p.h:156-190), given their adjoints
// la[12]; accumulates into ls, lm.
template <class R>
__device__ __forceinline__ void deposit_adjoint(R q, V3<R> s, V3<R> m, const R* la, V3<R>& ls, V3<R>& lm) {
  const R one = 1;
  R lcorr = 0;
  auto block = [&](R qs, R da, R db, const R* A, R& lqs, R& lda, R& ldb) {
    const R w0 = (one - da) * (one - db), w1 = (one + da) * (one - db);
    const R w2 = (one - da) * (one + db), w3 = (one + da) * (one + db);
    lqs = A[0] * w0 + A[1] * w1 + A[2] * w2 + A[3] * w3;
    lda += qs * (-A[0] * (one - db) + A[1] * (one - db) - A[2] * (one + db) + A[3] * (one + db));
    ldb += qs * (-A[0] * (one - da) - A[1] * (one + da) + A[2] * (one - da) + A[3] * (one + da));
    lcorr += A[0] - A[1] - A[2] + A[3];
  };
  R lqx, lqy, lqz;
  block(q * s.x, m.y, m.z, la + 0, lqx, lm.y, lm.z);  // jx: CALC_J(x,y,z)
  block(q * s.y, m.z, m.x, la + 4, lqy, lm.z, lm.x);  // jy: CALC_J(y,z,x)
  block(q * s.z, m.x, m.y, la + 8, lqz, lm.x, lm.y);  // jz: CALC_J(z,x,y)
  const R third = R(1) / R(3);
  ls.x += q * lqx + lcorr * q * s.y * s.z * third;
  ls.y += q * lqy + lcorr * q * s.x * s.z * third;
  ls.z += q * lqz + lcorr * q * s.x * s.y * third;
}

template <class R>
__device__ __forceinline__ R comp(const V3<R>& v, int a) { return a == 0 ? v.x : (a == 1 ? v.y : v.z); }
template <class R>
__device__ __forceinline__ void set_comp(V3<R>& v, int a, R val) {
  if (a == 0) v.x = val; else if (a == 1) v.y = val; else v.z = val;
}

// One streak of the forward split (move_p.h:93-371; an in-cell move is one
// streak with axis 3): from the streak's start (pos, rem, c) returns its
// half-length `len` and face `axis`, and advances (pos, rem, c) to the next
// streak's start.
template <class R>
__device__ __forceinline__ void streak_step(V3<R>& pos, V3<R>& rem, int& c, bool inb, const GridDev& g,
                                            R& len, int& axis) {
  axis = 3;
  len = 2;
  if (!inb) {
    for (int ax = 0; ax < 3; ++ax) {
      const R r = comp(rem, ax);
      const R dir = r > 0 ? R(1) : R(-1);
      const R fr = (r == 0) ? R(3.4e38) : (dir - comp(pos, ax)) / r;
      if (fr < len) { len = fr; axis = ax; }
    }
  }
  len *= R(0.5);
  const V3<R> s{rem.x * len, rem.y * len, rem.z * len};
  // the face direction is the sign of the remaining displacement (move_p.h:109-111)
  const R dir = axis < 3 && comp(rem, axis) > 0 ? R(1) : R(-1);
  rem = {rem.x - s.x, rem.y - s.y, rem.z - s.z};
  pos = {pos.x + s.x + s.x, pos.y + s.y + s.y, pos.z + s.z + s.z};
  if (axis == 3) return;
  int ix = c, iy, iz;  // RANK_TO_INDEX (src/types.h:184-193)
  iy = div_magic(ix, g.dsx); ix -= iy * g.sx;
  iz = div_magic(iy, g.dsy); iy -= iz * g.sy;
  const int step = dir > 0 ? 1 : -1;
  if (axis == 0) ix += step; else if (axis == 1) iy += step; else iz += step;
  if (ix == 0) ix = g.nx; else if (ix == g.nx + 1) ix = 1;
  if (iy == 0) iy = g.ny; else if (iy == g.ny + 1) iy = 1;
  if (iz == 0) iz = g.nz; else if (iz == g.nz + 1) iz = 1;
  c = g.vox(ix, iy, iz);
  set_comp(pos, axis, -dir);
}

// The forward Boris step and displacement (push.h:124-182) with every
// intermediate the reverse sweep needs.
template <class R>
struct BorisFwd {
  V3<R> ha, cb, u1, c1, t, c2, u3, cu, d;
  R g1, b0, b1, b2, P, b3, D, b4, g3, rg;
};

template <class R, bool LITERAL>
__device__ __forceinline__ BorisFwd<R> boris_fwd(const R f[18], V3<R> x0, V3<R> u0, const AdjArgs<R>& a) {
  const R one = 1, k = a.qdt_2mc;
  BorisFwd<R> b;
  b.ha = {k * ((f[0] + x0.y * f[1]) + x0.z * (f[2] + x0.y * f[3])),
          k * ((f[4] + x0.z * f[5]) + x0.x * (f[6] + x0.z * f[7])),
          k * ((f[8] + x0.x * f[9]) + x0.y * (f[10] + x0.x * f[11]))};
  b.cb = {f[12] + x0.x * f[13], f[14] + x0.y * f[15], f[16] + x0.z * f[17]};
  b.u1 = {u0.x + b.ha.x, u0.y + b.ha.y, u0.z + b.ha.z};
  b.g1 = one + dot(b.u1, b.u1);
  b.b0 = k / root<R, LITERAL>(b.g1);
  b.b1 = dot(b.cb, b.cb);
  b.b2 = (b.b0 * b.b0) * b.b1;
  b.P = one + b.b2 * (R(1. / 3.) + b.b2 * R(2. / 15.));
  b.b3 = b.b0 * b.P;
  b.D = one + b.b1 * (b.b3 * b.b3);
  b.b4 = R(2) * b.b3 / b.D;
  b.c1 = cross(b.u1, b.cb);
  b.t = {b.u1.x + b.b3 * b.c1.x, b.u1.y + b.b3 * b.c1.y, b.u1.z + b.b3 * b.c1.z};
  b.c2 = cross(b.t, b.cb);
  b.u3 = {b.u1.x + b.b4 * b.c2.x + b.ha.x, b.u1.y + b.b4 * b.c2.y + b.ha.y, b.u1.z + b.b4 * b.c2.z + b.ha.z};
  b.g3 = one + dot(b.u3, b.u3);
  b.rg = one / root<R, LITERAL>(b.g3);
  b.cu = {b.u3.x * a.cdt_dx, b.u3.y * a.cdt_dy, b.u3.z * a.cdt_dz};
  b.d = {b.cu.x * b.rg, b.cu.y * b.rg, b.cu.z * b.rg};
  return b;
}

// A load the compiler cannot merge with an earlier load of the same address:
// the coefficients are read again after the streak sweep instead of being
// held in registers across it.
__device__ __forceinline__ float reload(const float* p) {
  float v;
  asm volatile("ld.global.nc.f32 %0, [%1];" : "=f"(v) : "l"(p));
  return v;
}
__device__ __forceinline__ double reload(const double* p) {
  double v;
  asm volatile("ld.global.nc.f64 %0, [%1];" : "=d"(v) : "l"(p));
  return v;
}

// The adjoint of one particle's push.  Writes lambda_x, lambda_u in place and
// returns the 18 interpolator adjoints of its cell in lf; false (nothing
// written, lf unset) for a particle the kernel cannot take.
template <class R, int VL, bool LITERAL>
__device__ __forceinline__ bool adjoint_one(const unsigned char* __restrict__ part, int64_t p,
                                            const R* __restrict__ interp, const R* __restrict__ lacc,
                                            unsigned char* __restrict__ lpart, const AdjArgs<R>& a,
                                            int* __restrict__ status, int& cell, R lf[18]) {
  using L = PLayout<R, VL>;
  auto mem = [&](const unsigned char* b, int m) { return *reinterpret_cast<const R*>(b + L::off(p, m)); };
  const V3<R> x0{mem(part, 0), mem(part, 1), mem(part, 2)};
  const V3<R> u0{mem(part, 3), mem(part, 4), mem(part, 5)};
  const R w = mem(part, 6);
  cell = *reinterpret_cast<const int*>(part + L::cell_off(p));
  const V3<R> lxo{mem(lpart, 0), mem(lpart, 1), mem(lpart, 2)};
  const V3<R> luo{mem(lpart, 3), mem(lpart, 4), mem(lpart, 5)};
  if ((unsigned)cell >= (unsigned)a.g.num_cells) {
    atomicOr(status, CPIC_STATUS_CELL_RANGE);
    return false;
  }
  const R one = 1, k = a.qdt_2mc;
  R f[18];
#pragma unroll
  for (int m = 0; m < 18; ++m) f[m] = __ldg(interp + cell_at<18>(cell, m));

  // ---------------- forward recompute (push.h:124-182): only the
  // displacement is kept through the streak sweep; the Boris intermediates
  // are recomputed after it (fewer live registers, more resident warps)
  V3<R> d;
  {
    const BorisFwd<R> fw = boris_fwd<R, LITERAL>(f, x0, u0, a);
    d = fw.d;
  }
  const R q = w * a.qsp;

  // streak split: count the streaks (their states are replayed in reverse)
  const V3<R> np{x0.x + R(2) * d.x, x0.y + R(2) * d.y, x0.z + R(2) * d.z};
  const bool inb = np.x <= one && np.y <= one && np.z <= one && -np.x <= one && -np.y <= one &&
                   -np.z <= one;
  int ns = 0;
  {
    V3<R> pos = x0, rem = d;
    int c = cell;
    bool done = false;
    for (int it = 0; it < kMaxAdjStreaks; ++it) {
      R len;
      int axis;
      streak_step<R>(pos, rem, c, inb, a.g, len, axis);
      ++ns;
      if (axis == 3) { done = true; break; }
    }
    if (!done) {
      atomicOr(status, CPIC_STATUS_MOVER_CAP);
      return false;
    }
  }

  // ---------------- reverse: streaks (last to first), each replayed from the start
  V3<R> lpos = lxo, lrem{0, 0, 0};
  for (int kk = ns - 1; kk >= 0; --kk) {
    V3<R> pos = x0, rem = d;
    int c = cell;
    R len;
    int ax;
    for (int j = 0; j < kk; ++j) streak_step<R>(pos, rem, c, inb, a.g, len, ax);
    {
      V3<R> pos1 = pos, rem1 = rem;
      int c1 = c;
      streak_step<R>(pos1, rem1, c1, inb, a.g, len, ax);
    }
    const V3<R> s{rem.x * len, rem.y * len, rem.z * len};
    const V3<R> mid{pos.x + s.x, pos.y + s.y, pos.z + s.z};
    V3<R> ls{0, 0, 0}, lm{0, 0, 0}, lp{0, 0, 0};
    // pos' = pos + 2 s, except the crossed axis, which is set to a constant
    for (int b = 0; b < 3; ++b) {
      if (b == ax) continue;
      set_comp(lp, b, comp(lpos, b));
      set_comp(ls, b, comp(ls, b) + R(2) * comp(lpos, b));
    }
    // rem' = rem - s
    V3<R> lr = lrem;
    ls = {ls.x - lrem.x, ls.y - lrem.y, ls.z - lrem.z};
    // deposit of the streak into its cell
    R la[12];
    {
      const R* ap = lacc + (size_t)c * 12;
#pragma unroll
      for (int m = 0; m < 12; ++m) la[m] = __ldg(ap + m);
    }
    deposit_adjoint<R>(q, s, mid, la, ls, lm);
    // mid = pos + s
    lp = {lp.x + lm.x, lp.y + lm.y, lp.z + lm.z};
    ls = {ls.x + lm.x, ls.y + lm.y, ls.z + lm.z};
    // s = rem * len
    lr = {lr.x + ls.x * len, lr.y + ls.y * len, lr.z + ls.z * len};
    const R llen = dot(ls, rem);
    if (ax < 3) {  // len = (dir - pos_ax) / (2 rem_ax)
      const R r = comp(rem, ax);
      set_comp(lp, ax, comp(lp, ax) - llen * R(0.5) / r);
      set_comp(lr, ax, comp(lr, ax) - llen * len / r);
    }
    lpos = lp;
    lrem = lr;
  }
  // lpos: adjoint of the starting offsets through the move; lrem: adjoint of d

  // ---------------- reverse: displacement and Boris (push.h:144-182)
#pragma unroll
  for (int m = 0; m < 18; ++m) f[m] = reload(interp + cell_at<18>(cell, m));
  const BorisFwd<R> fw = boris_fwd<R, LITERAL>(f, x0, u0, a);
  const V3<R> ha = fw.ha, cb = fw.cb, u1 = fw.u1, c1 = fw.c1, t = fw.t, c2 = fw.c2, u3 = fw.u3, cu = fw.cu;
  const R g1 = fw.g1, b0 = fw.b0, b1 = fw.b1, b2 = fw.b2, P = fw.P, b3 = fw.b3, D = fw.D, b4 = fw.b4;
  const R g3 = fw.g3, rg = fw.rg;
  (void)ha;
  V3<R> lx = lpos;
  V3<R> lu3{luo.x + lrem.x * a.cdt_dx * rg, luo.y + lrem.y * a.cdt_dy * rg, luo.z + lrem.z * a.cdt_dz * rg};
  const R lrg = dot(lrem, cu);
  const R lg3 = R(-0.5) * rg / g3 * lrg;
  lu3 = {lu3.x + R(2) * u3.x * lg3, lu3.y + R(2) * u3.y * lg3, lu3.z + R(2) * u3.z * lg3};
  V3<R> lha = lu3;  // u3 = u2 + ha
  V3<R> lu1 = lu3;  // u2 = u1 + b4 (t x cb)
  const R lb4 = dot(lu3, c2);
  const V3<R> v{b4 * lu3.x, b4 * lu3.y, b4 * lu3.z};
  V3<R> lt = cross(cb, v);
  V3<R> lcb = cross(v, t);
  // t = u1 + b3 (u1 x cb)
  const V3<R> wv{b3 * lt.x, b3 * lt.y, b3 * lt.z};
  const V3<R> cw = cross(cb, wv);
  lu1 = {lu1.x + lt.x + cw.x, lu1.y + lt.y + cw.y, lu1.z + lt.z + cw.z};
  R lb3 = dot(lt, c1);
  const V3<R> wu = cross(wv, u1);
  lcb = {lcb.x + wu.x, lcb.y + wu.y, lcb.z + wu.z};
  // b4 = 2 b3 / D, D = 1 + b1 b3^2
  lb3 += lb4 * R(2) * (one / D - R(2) * b1 * b3 * b3 / (D * D));
  R lb1 = lb4 * (R(-2) * b3 * b3 * b3 / (D * D));
  // b3 = b0 P(b2)
  R lb0 = lb3 * P;
  const R lb2 = lb3 * b0 * (R(1. / 3.) + R(4. / 15.) * b2);
  // b2 = b0^2 b1
  lb0 += lb2 * R(2) * b0 * b1;
  lb1 += lb2 * b0 * b0;
  // b1 = |cb|^2
  lcb = {lcb.x + R(2) * cb.x * lb1, lcb.y + R(2) * cb.y * lb1, lcb.z + R(2) * cb.z * lb1};
  // b0 = k / sqrt(g1)
  const R lg1 = R(-0.5) * b0 / g1 * lb0;
  lu1 = {lu1.x + R(2) * u1.x * lg1, lu1.y + R(2) * u1.y * lg1, lu1.z + R(2) * u1.z * lg1};
  // u1 = u0 + ha
  lha = {lha.x + lu1.x, lha.y + lu1.y, lha.z + lu1.z};

  // ---------------- reverse: field at the particle (push.h:124-138)
  lf[0] = k * lha.x;
  lf[1] = k * x0.y * lha.x;
  lf[2] = k * x0.z * lha.x;
  lf[3] = k * x0.y * x0.z * lha.x;
  lx.y += k * (f[1] + x0.z * f[3]) * lha.x;
  lx.z += k * (f[2] + x0.y * f[3]) * lha.x;
  lf[4] = k * lha.y;
  lf[5] = k * x0.z * lha.y;
  lf[6] = k * x0.x * lha.y;
  lf[7] = k * x0.x * x0.z * lha.y;
  lx.z += k * (f[5] + x0.x * f[7]) * lha.y;
  lx.x += k * (f[6] + x0.z * f[7]) * lha.y;
  lf[8] = k * lha.z;
  lf[9] = k * x0.x * lha.z;
  lf[10] = k * x0.y * lha.z;
  lf[11] = k * x0.x * x0.y * lha.z;
  lx.x += k * (f[9] + x0.y * f[11]) * lha.z;
  lx.y += k * (f[10] + x0.x * f[11]) * lha.z;
  lf[12] = lcb.x; lf[13] = x0.x * lcb.x; lx.x += f[13] * lcb.x;
  lf[14] = lcb.y; lf[15] = x0.y * lcb.y; lx.y += f[15] * lcb.y;
  lf[16] = lcb.z; lf[17] = x0.z * lcb.z; lx.z += f[17] * lcb.z;

  // adjoint before the step, in place
  auto put = [&](int m, R v) { *reinterpret_cast<R*>(lpart + L::off(p, m)) = v; };
  put(0, lx.x); put(1, lx.y); put(2, lx.z);
  put(3, lu1.x); put(4, lu1.y); put(5, lu1.z);
  return true;
}

// Sum of v[0..17] over the 32 lanes, scattered: afterwards lane l holds the
// total of value index value18_of_lane(l) (18 lanes hold distinct values).
// Halving levels over 18 -> 9 -> 5 -> 3 -> 2 -> 1 values (odd counts padded
// with a zero): 20 shuffles.
template <class R>
__device__ __forceinline__ R reduce_scatter18(const R v[18], int lane) {
  const bool h16 = lane & 16, h8 = lane & 8, h4 = lane & 4, h2 = lane & 2, h1 = lane & 1;
  R a9[9];
#pragma unroll
  for (int k = 0; k < 9; ++k)
    a9[k] = (h16 ? v[k + 9] : v[k]) + __shfl_xor_sync(kFull, h16 ? v[k] : v[k + 9], 16);
  R b5[5];
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    const R hi = k + 5 < 9 ? a9[k + 5] : R(0);
    b5[k] = (h8 ? hi : a9[k]) + __shfl_xor_sync(kFull, h8 ? a9[k] : hi, 8);
  }
  R c3[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const R hi = k + 3 < 5 ? b5[k + 3] : R(0);
    c3[k] = (h4 ? hi : b5[k]) + __shfl_xor_sync(kFull, h4 ? b5[k] : hi, 4);
  }
  R d2[2];
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const R hi = k + 2 < 3 ? c3[k + 2] : R(0);
    d2[k] = (h2 ? hi : c3[k]) + __shfl_xor_sync(kFull, h2 ? c3[k] : hi, 2);
  }
  return (h1 ? d2[1] : d2[0]) + __shfl_xor_sync(kFull, h1 ? d2[0] : d2[1], 1);
}

// Value index held by `lane` after reduce_scatter18, or -1.
__device__ __forceinline__ int value18_of_lane(int lane) {
  const int i4 = 2 * ((lane >> 1) & 1) + (lane & 1);
  if (i4 >= 3) return -1;
  const int i3 = 3 * ((lane >> 2) & 1) + i4;
  if (i3 >= 5) return -1;
  const int i2 = 5 * ((lane >> 3) & 1) + i3;
  if (i2 >= 9) return -1;
  return 9 * ((lane >> 4) & 1) + i2;
}

// 8 consecutive bytes of float (red.global.add.v2.f32; 8-byte aligned).
__device__ __forceinline__ void red_add2(float* a, float v0, float v1) {
  asm volatile("red.global.add.v2.f32 [%0], {%1,%2};" ::"l"(a), "f"(v0), "f"(v1) : "memory");
}

// Adds the 18 coefficient adjoints of one particle to its cell's row (ROWS
// layout): 4 x 16 + 8 bytes of vector reductions for float, scalar atomics
// over 144 consecutive bytes for double.
__device__ __forceinline__ void red_row18(float* row, const float v[18]) {
#pragma unroll
  for (int k = 0; k < 4; ++k) red_add4(row + 4 * k, v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]);
  red_add2(row + 16, v[16], v[17]);
}
__device__ __forceinline__ void red_row18(double* row, const double v[18]) {
#pragma unroll
  for (int m = 0; m < 18; ++m) red_add(row + m, v[m]);
}

// ROWS: lambda_interp in cell-major rows of CPIC_ADJ_INTERP_ROW values.
template <class R, int VL, bool LITERAL, bool ROWS>
__global__ void __launch_bounds__(kAdjThreads)
adjoint_push_kernel(const unsigned char* __restrict__ part, int n, const R* __restrict__ interp,
                    const R* __restrict__ lacc, unsigned char* __restrict__ lpart, R* __restrict__ linterp,
                    const AdjArgs<R> a, int* __restrict__ status) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = (int)(threadIdx.x & 31);
  R lf[18];
  int cell = 0;
  const bool dep = p < n && adjoint_one<R, VL, LITERAL>(part, p, interp, lacc, lpart, a, status, cell, lf);
  // transpose of the gather: the largest group of lanes sharing a cell is
  // reduced over the warp (18 atomics for the group), the others add their own
  const int key = dep ? cell : -1 - lane;
  const unsigned peers = __match_any_sync(kFull, key);
  const unsigned score = dep ? ((unsigned)__popc(peers) << 5) | (unsigned)(31 - (__ffs(peers) - 1)) : 0u;
  const unsigned best = __reduce_max_sync(kFull, score);
  const int bsize = (int)(best >> 5);
  const int leader = 31 - (int)(best & 31);
  bool in_major = false;
  if (bsize >= 2) {  // warp-uniform
    in_major = dep && ((peers >> leader) & 1u);
    R w[18];
#pragma unroll
    for (int m = 0; m < 18; ++m) w[m] = in_major ? lf[m] : R(0);
    const R tot = reduce_scatter18<R>(w, lane);
    const int major_cell = __shfl_sync(kFull, cell, leader);
    const int vi = value18_of_lane(lane);
    if (vi >= 0)
      red_add(linterp + (ROWS ? (size_t)major_cell * CPIC_ADJ_INTERP_ROW + vi : cell_at<18>(major_cell, vi)), tot);
  }
  if (dep && !in_major) {
    if constexpr (ROWS) {
      red_row18(linterp + (size_t)cell * CPIC_ADJ_INTERP_ROW, lf);
    } else {
#pragma unroll
      for (int m = 0; m < 18; ++m) red_add(linterp + cell_at<18>(cell, m), lf[m]);
    }
  }
}

template <class R, int VL, bool LITERAL>
int launch_adjoint(const void* part, int n, const void* interp, const void* lacc, void* lpart, void* linterp,
                   const AdjArgs<R>& a, int* status, cudaStream_t s, bool rows) {
  const unsigned blocks = (unsigned)(((int64_t)n + kAdjThreads - 1) / kAdjThreads);
  if (rows)
    adjoint_push_kernel<R, VL, LITERAL, true><<<blocks, kAdjThreads, 0, s>>>(
        static_cast<const unsigned char*>(part), n, static_cast<const R*>(interp), static_cast<const R*>(lacc),
        static_cast<unsigned char*>(lpart), static_cast<R*>(linterp), a, status);
  else
    adjoint_push_kernel<R, VL, LITERAL, false><<<blocks, kAdjThreads, 0, s>>>(
        static_cast<const unsigned char*>(part), n, static_cast<const R*>(interp), static_cast<const R*>(lacc),
        static_cast<unsigned char*>(lpart), static_cast<R*>(linterp), a, status);
  return launch_status();
}

template <class R>
int adjoint_typed(const void* part, int n, const void* interp, const void* lacc, void* lpart, void* linterp,
                  const cpic_grid* g, const cpic_push_params* prm, int* status, cudaStream_t s) {
  AdjArgs<R> a{(R)prm->qdt_2mc, (R)prm->cdt_dx, (R)prm->cdt_dy, (R)prm->cdt_dz, (R)prm->qsp, make_grid(g)};
  const bool literal = !(prm->flags & CPIC_PUSH_TRUE_SQRT) && sizeof(R) == 8;
  const bool rows = (prm->flags & CPIC_ADJ_INTERP_ROWS) != 0;
  if (prm->particle_vl == 32)
    return literal ? launch_adjoint<R, 32, true>(part, n, interp, lacc, lpart, linterp, a, status, s, rows)
                   : launch_adjoint<R, 32, false>(part, n, interp, lacc, lpart, linterp, a, status, s, rows);
  return literal ? launch_adjoint<R, 16, true>(part, n, interp, lacc, lpart, linterp, a, status, s, rows)
                 : launch_adjoint<R, 16, false>(part, n, interp, lacc, lpart, linterp, a, status, s, rows);
}

}  // namespace
}  // namespace cpic

extern "C" int cpic_adjoint_push(const void* particles, int64_t num_particles, const void* interpolators,
                                 const void* lambda_acc, void* lambda_particles, void* lambda_interp,
                                 const cpic_grid* grid, const cpic_push_params* prm, int32_t* d_status,
                                 cpic_stream_t stream) {
  using namespace cpic;
  if (!grid || !prm || !d_status) return CPIC_EINVAL;
  int rc = check_grid(grid);
  if (rc) return rc;
  if (num_particles < 0 || num_particles > 0x7fffffffLL - 64) return CPIC_EINVAL;
  if (prm->precision != CPIC_FLOAT && prm->precision != CPIC_DOUBLE) return CPIC_EINVAL;
  if (prm->particle_vl != 16 && prm->particle_vl != 32) return CPIC_EINVAL;
  if (prm->flags & ~(CPIC_PUSH_TRUE_SQRT | CPIC_PUSH_EXACT | CPIC_ADJ_INTERP_ROWS)) return CPIC_EINVAL;
  if (num_particles == 0) return CPIC_OK;
  if (!particles || !interpolators || !lambda_acc || !lambda_particles || !lambda_interp) return CPIC_EINVAL;
  // the row layout's vector reductions need 16-byte aligned rows
  if ((prm->flags & CPIC_ADJ_INTERP_ROWS) && ((uintptr_t)lambda_interp & 15)) return CPIC_EINVAL;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const int n = (int)num_particles;
  if (prm->precision == CPIC_FLOAT)
    return adjoint_typed<float>(particles, n, interpolators, lambda_acc, lambda_particles, lambda_interp, grid,
                                prm, d_status, s);
  return adjoint_typed<double>(particles, n, interpolators, lambda_acc, lambda_particles, lambda_interp, grid,
                               prm, d_status, s);
}
