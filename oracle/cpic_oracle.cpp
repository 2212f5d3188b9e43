// cpic_oracle.cpp -- CPU restatement of CabanaPIC's per-step hot path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the parity oracle: the tests, the
// smoke check and the CPU-baseline leg of the benchmark load it as the oracle.
// Nothing in the shipped library (cabanapic_gb300/) links, loads or calls it.
//
// Parity pin: the oracle reproduces the reference's own golden energy histories
// (tests/energy_comparison/energies_gold.2stream-em.{float,double}) for the
// 2stream-em deck, see tests/test_oracle_gold.py.
//
// Every routine follows the reference's arithmetic operation by operation (same
// operand order, same literal types), because bit parity with a real_t build of
// the reference depends on it.  The code structure is this project's own.
// Build recipe: oracle/build.py (g++ -O3 -ffp-contract=off -fopenmp).
//
// Layouts (the reference's ABI, see src/types.h in the reference):
//   particles     Cabana AoSoA<real_t x7, int>, vector length VL (runtime here):
//                 SoA block s holds members [x y z ux uy uz w](VL each) then cell[VL]
//   interpolators AoSoA<real_t x18>, VL = 32  (src/types.h:64-108)
//   fields        AoSoA<real_t x9>,  VL = 32  (src/types.h:138-172)
//   accumulators  View<real_t*[3][4]>, LayoutRight: [cell][comp][quadrant]

#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace orc {

constexpr int kCellBlock = 32;  // CELL_BLOCK_FACTOR, src/types.h:15-17
enum { kInterpMembers = 18, kFieldMembers = 9 };
enum Interp { EX = 0, DEXDY, DEXDZ, D2EXDYDZ, EY, DEYDZ, DEYDX, D2EYDZDX,
              EZ, DEZDX, DEZDY, D2EZDXDY, CBX, DCBXDX, CBY, DCBYDY, CBZ, DCBZDZ };
enum Field { F_EX = 0, F_EY, F_EZ, F_CBX, F_CBY, F_CBZ, F_JFX, F_JFY, F_JFZ };
enum { JX = 0, JY = 1, JZ = 2 };

// ---------------------------------------------------------------- layouts
template <class R>
struct Particles {
  unsigned char* base;
  int vl;
  size_t block_bytes() const { return (size_t)vl * (7 * sizeof(R) + sizeof(int)); }
  R& mem(int m, size_t p) const {
    size_t s = p / vl, i = p % vl;
    return *reinterpret_cast<R*>(base + s * block_bytes() + ((size_t)m * vl + i) * sizeof(R));
  }
  int& cell(size_t p) const {
    size_t s = p / vl, i = p % vl;
    return *reinterpret_cast<int*>(base + s * block_bytes() + (size_t)7 * vl * sizeof(R) + i * sizeof(int));
  }
};

template <class R, int NM>
struct CellSoA {
  R* a;
  R& operator()(size_t c, int m) const {
    return a[(c / kCellBlock) * (size_t)(NM * kCellBlock) + (size_t)m * kCellBlock + c % kCellBlock];
  }
};

struct Grid {
  long nx, ny, nz, ng;
  long sx() const { return nx + 2 * ng; }
  long sy() const { return ny + 2 * ng; }
  long sz() const { return nz + 2 * ng; }
  long cells() const { return sx() * sy() * sz(); }
  // VOXEL macro, src/types.h:195
  long vox(long x, long y, long z) const { return x + sx() * (y + sy() * z); }
};

// Per-cell loops below run under OpenMP: every iteration writes only its own
// cell, so the results do not depend on the thread count.

// Accumulator sink: the reference scatter-adds into View<real_t*[3][4]>.  The
// optional abs/count arrays record, per (cell, comp, quadrant), the sum of
// |contribution| and the number of terms; the tests use them to bound the
// reordering error of the GPU's atomic summation.
template <class R>
struct AccSink {
  R* acc;
  R* abs_sum;   // may be null
  int* count;   // may be null
  void add(long cell, int comp, int q, R v) const {
    size_t k = (size_t)cell * 12 + comp * 4 + q;
    acc[k] += v;
    if (abs_sum) abs_sum[k] += std::fabs(v);
    if (count) count[k] += 1;
  }
};

// sqrt used by push for gamma.  The reference calls sqrtf() even when
// real_t=double (src/push.h:148,169); literal=true keeps that.
template <class R>
inline R gamma_sqrt(R arg, bool literal) {
  if (literal) return (R)sqrtf((float)arg);
  return (R)std::sqrt(arg);
}

// ---------------------------------------------------------------- deposit
// Four quadrant currents for one axis (src/push.h:218-232 and
// src/move_p.h:156-170 use the same sequence).  u = q-weighted displacement
// along the axis, da/db = offsets along the two transverse axes, corr = the
// q*ux*uy*uz/3 correction.
template <class R>
inline void quad_currents(R qu, R da, R db, R corr, R out[4]) {
  const R one = 1;
  R t = qu;
  R a1 = t * da;
  R a0 = t - a1;
  a1 += t;
  R s = one + db;
  R a2 = a0 * s;
  R a3 = a1 * s;
  s = one - db;
  a0 *= s;
  a1 *= s;
  a0 += corr;
  a1 -= corr;
  a2 -= corr;
  a3 += corr;
  out[0] = a0; out[1] = a1; out[2] = a2; out[3] = a3;
}

template <class R>
inline void deposit12(const AccSink<R>& sink, long cell, R q, R ux, R uy, R uz,
                      R dx, R dy, R dz, R corr) {
  R j[4];
  quad_currents<R>(q * ux, dy, dz, corr, j);  // CALC_J(x,y,z)
  for (int k = 0; k < 4; ++k) sink.add(cell, JX, k, j[k]);
  quad_currents<R>(q * uy, dz, dx, corr, j);  // CALC_J(y,z,x)
  for (int k = 0; k < 4; ++k) sink.add(cell, JY, k, j[k]);
  quad_currents<R>(q * uz, dx, dy, corr, j);  // CALC_J(z,x,y)
  for (int k = 0; k < 4; ++k) sink.add(cell, JZ, k, j[k]);
}

// ---------------------------------------------------------------- move_p
// Cell-crossing mover, src/move_p.h:59-374 with detect_leaving_domain
// (src/move_p.h:9-54).  Periodic boundary only.  Returns the number of streaks.
template <class R>
int move_particle(const Particles<R>& P, size_t p, R q, R disp[3],
                  const AccSink<R>& sink, const Grid& g) {
  int streaks = 0;
  for (;;) {
    ++streaks;
    R mid[3] = {P.mem(0, p), P.mem(1, p), P.mem(2, p)};
    R sd[3] = {disp[0], disp[1], disp[2]};
    R dir[3];
    for (int a = 0; a < 3; ++a) dir[a] = (sd[a] > 0) ? 1 : -1;
    // twice the fractional distance to each face; double sentinel (move_p.h:115-117)
    R frac[3];
    for (int a = 0; a < 3; ++a) frac[a] = (sd[a] == 0) ? 3.4e38 : (dir[a] - mid[a]) / sd[a];
    R len = 2;
    int axis = 3;
    for (int a = 0; a < 3; ++a)
      if (frac[a] < len) { len = frac[a]; axis = a; }
    len *= 0.5;
    for (int a = 0; a < 3; ++a) sd[a] *= len;
    for (int a = 0; a < 3; ++a) mid[a] += sd[a];

    long ii = P.cell(p);
    // correction uses a double 1/3 literal here (move_p.h:154)
    R corr = q * sd[0] * sd[1] * sd[2] * (1. / 3.);
    deposit12<R>(sink, ii, q, sd[0], sd[1], sd[2], mid[0], mid[1], mid[2], corr);

    for (int a = 0; a < 3; ++a) disp[a] -= sd[a];
    for (int a = 0; a < 3; ++a) P.mem(a, p) += sd[a] + sd[a];
    if (axis == 3) break;

    R face_sign = dir[axis];
    P.mem(axis, p) = face_sign;  // land exactly on the face
    int face = axis + (face_sign > 0 ? 3 : 0);

    // RANK_TO_INDEX (types.h:184-193) on the ghosted extents
    int X = (int)g.sx(), Y = (int)g.sy();
    int ix = (int)ii, iy, iz;
    iy = ix / X; ix -= iy * X;
    iz = iy / Y; iy -= iz * Y;
    long c[3] = {ix, iy, iz};
    if (face < 3) c[face] -= 1; else c[face - 3] += 1;

    // detect_leaving_domain: the last matching test wins
    int leaving = -1;
    if (c[0] == 0) leaving = 0;
    if (c[1] == 0) leaving = 1;
    if (c[2] == 0) leaving = 2;
    if (c[0] == g.nx + 1) leaving = 3;
    if (c[1] == g.ny + 1) leaving = 4;
    if (c[2] == g.nz + 1) leaving = 5;
    if (leaving >= 0) {  // periodic wrap (move_p.h:271-288)
      if (leaving == 0) c[0] = (g.nx - 1) + g.ng;
      else if (leaving == 1) c[1] = (g.ny - 1) + g.ng;
      else if (leaving == 2) c[2] = (g.nz - 1) + g.ng;
      else if (leaving == 3) c[0] = g.ng;
      else if (leaving == 4) c[1] = g.ng;
      else c[2] = g.ng;
    }
    P.cell(p) = (int)g.vox(c[0], c[1], c[2]);
    P.mem(axis, p) = -face_sign;  // convert coordinate system
  }
  return streaks;
}

// ---------------------------------------------------------------- push
// One particle of push(), src/push.h:66-295.
template <class R>
inline void push_one(const Particles<R>& P, size_t p, const CellSoA<R, kInterpMembers>& f,
                     R qdt_2mc, R cdt_dx, R cdt_dy, R cdt_dz, R qsp,
                     const AccSink<R>& sink, const Grid& g, bool literal, long* crossers) {
  const R one = 1.;
  const R one_third = 1. / 3.;
  const R two_fifteenths = 2. / 15.;
  long ii = P.cell(p);
  R ex = f(ii, EX), dexdy = f(ii, DEXDY), dexdz = f(ii, DEXDZ), d2exdydz = f(ii, D2EXDYDZ);
  R ey = f(ii, EY), deydz = f(ii, DEYDZ), deydx = f(ii, DEYDX), d2eydzdx = f(ii, D2EYDZDX);
  R ez = f(ii, EZ), dezdx = f(ii, DEZDX), dezdy = f(ii, DEZDY), d2ezdxdy = f(ii, D2EZDXDY);
  R cbx = f(ii, CBX), dcbxdx = f(ii, DCBXDX), cby = f(ii, CBY), dcbydy = f(ii, DCBYDY);
  R cbz = f(ii, CBZ), dcbzdz = f(ii, DCBZDZ);

  R dx = P.mem(0, p), dy = P.mem(1, p), dz = P.mem(2, p);
  // field at the particle (push.h:124-138)
  R hax = qdt_2mc * ((ex + dy * dexdy) + dz * (dexdz + dy * d2exdydz));
  R hay = qdt_2mc * ((ey + dz * deydz) + dx * (deydx + dz * d2eydzdx));
  R haz = qdt_2mc * ((ez + dx * dezdx) + dy * (dezdy + dx * d2ezdxdy));
  cbx = cbx + dx * dcbxdx;
  cby = cby + dy * dcbydy;
  cbz = cbz + dz * dcbzdz;

  R ux = P.mem(3, p), uy = P.mem(4, p), uz = P.mem(5, p);
  ux += hax; uy += hay; uz += haz;
  // relativistic Boris rotation (push.h:148-163)
  R b0 = qdt_2mc / gamma_sqrt<R>(one + (ux * ux + (uy * uy + uz * uz)), literal);
  R b1 = cbx * cbx + (cby * cby + cbz * cbz);
  R b2 = (b0 * b0) * b1;
  R b3 = b0 * (one + b2 * (one_third + b2 * two_fifteenths));
  R b4 = b3 / (one + b1 * (b3 * b3));
  b4 += b4;
  R px = ux + b3 * (uy * cbz - uz * cby);
  R py = uy + b3 * (uz * cbx - ux * cbz);
  R pz = uz + b3 * (ux * cby - uy * cbx);
  ux += b4 * (py * cbz - pz * cby);
  uy += b4 * (pz * cbx - px * cbz);
  uz += b4 * (px * cby - py * cbx);
  ux += hax; uy += hay; uz += haz;
  P.mem(3, p) = ux; P.mem(4, p) = uy; P.mem(5, p) = uz;

  // normalised half displacement (push.h:169-182)
  R rg = one / gamma_sqrt<R>(one + (ux * ux + (uy * uy + uz * uz)), literal);
  ux *= cdt_dx; uy *= cdt_dy; uz *= cdt_dz;
  ux *= rg; uy *= rg; uz *= rg;
  R mx = dx + ux, my = dy + uy, mz = dz + uz;   // streak midpoint
  R nx = mx + ux, ny = my + uy, nz = mz + uz;   // new position
  R q = P.mem(6, p) * qsp;

  if (nx <= one && ny <= one && nz <= one && -nx <= one && -ny <= one && -nz <= one) {
    P.mem(0, p) = nx; P.mem(1, p) = ny; P.mem(2, p) = nz;
    R corr = q * ux * uy * uz * one_third;
    deposit12<R>(sink, ii, q, ux, uy, uz, mx, my, mz, corr);
  } else {
    R disp[3] = {ux, uy, uz};
    move_particle<R>(P, p, q, disp, sink, g);
    if (crossers) ++*crossers;
  }
}

template <class R>
void push_serial(const Particles<R>& P, size_t n, const R* interp, R qdt_2mc, R cdt_dx,
                 R cdt_dy, R cdt_dz, R qsp, const AccSink<R>& sink, const Grid& g,
                 bool literal, long* crossers) {
  CellSoA<R, kInterpMembers> f{const_cast<R*>(interp)};
  for (size_t p = 0; p < n; ++p)
    push_one<R>(P, p, f, qdt_2mc, cdt_dx, cdt_dy, cdt_dz, qsp, sink, g, literal, crossers);
}

// OpenMP push with one private accumulator copy per thread, summed after the
// loop: the semantics of Kokkos' duplicated ScatterView on the OpenMP backend
// (example/example.cpp:139,248,251).  Used as the timed CPU baseline.
template <class R>
void push_openmp(const Particles<R>& P, size_t n, const R* interp, R qdt_2mc, R cdt_dx,
                 R cdt_dy, R cdt_dz, R qsp, R* acc, const Grid& g, bool literal,
                 int threads, std::vector<R>& dup) {
  CellSoA<R, kInterpMembers> f{const_cast<R*>(interp)};
  size_t acc_len = (size_t)g.cells() * 12;
#ifdef _OPENMP
  if (threads <= 0) threads = omp_get_max_threads();
#else
  threads = 1;
#endif
  if (dup.size() < acc_len * (size_t)threads) dup.assign(acc_len * (size_t)threads, R(0));
#pragma omp parallel num_threads(threads)
  {
    int t = 0;
#ifdef _OPENMP
    t = omp_get_thread_num();
#endif
    R* mine = dup.data() + (size_t)t * acc_len;
    // reset of the private copy (ScatterView::reset_except)
    std::memset(mine, 0, acc_len * sizeof(R));
    AccSink<R> sink{mine, nullptr, nullptr};
    size_t blocks = (n + P.vl - 1) / P.vl;
#pragma omp for schedule(static)
    for (long s = 0; s < (long)blocks; ++s) {
      size_t p0 = (size_t)s * P.vl, p1 = p0 + P.vl < n ? p0 + P.vl : n;
      for (size_t p = p0; p < p1; ++p)
        push_one<R>(P, p, f, qdt_2mc, cdt_dx, cdt_dy, cdt_dz, qsp, sink, g, literal, nullptr);
    }
    // contribute: sum the copies into the target accumulator
#pragma omp for schedule(static)
    for (long k = 0; k < (long)acc_len; ++k) {
      R s = acc[k];
      for (int u = 0; u < threads; ++u) s += dup[(size_t)u * acc_len + k];
      acc[k] = s;
    }
  }
}

// ---------------------------------------------------------------- uncenter
// uncenter_particles, src/uncenter_p.h:4-105: Boris rotation with
// qdt_4mc = -0.5*qdt_2mc, then the half E kick (in that order, as written).
template <class R>
void uncenter(const Particles<R>& P, size_t n, const R* interp, R qdt_2mc) {
  CellSoA<R, kInterpMembers> f{const_cast<R*>(interp)};
  const R qdt_4mc = -0.5 * qdt_2mc;
  const R one = 1.;
  const R one_third = 1. / 3.;
  const R two_fifteenths = 2. / 15.;
  for (size_t p = 0; p < n; ++p) {
    R dx = P.mem(0, p), dy = P.mem(1, p), dz = P.mem(2, p);
    long ii = P.cell(p);
    R hax = qdt_2mc * ((f(ii, EX) + dy * f(ii, DEXDY)) + dz * (f(ii, DEXDZ) + dy * f(ii, D2EXDYDZ)));
    R hay = qdt_2mc * ((f(ii, EY) + dz * f(ii, DEYDZ)) + dx * (f(ii, DEYDX) + dz * f(ii, D2EYDZDX)));
    R haz = qdt_2mc * ((f(ii, EZ) + dx * f(ii, DEZDX)) + dy * (f(ii, DEZDY) + dx * f(ii, D2EZDXDY)));
    R cbx = f(ii, CBX) + dx * f(ii, DCBXDX);
    R cby = f(ii, CBY) + dy * f(ii, DCBYDY);
    R cbz = f(ii, CBZ) + dz * f(ii, DCBZDZ);
    R ux = P.mem(3, p), uy = P.mem(4, p), uz = P.mem(5, p);
    // (real_t)sqrt(real_t): exact as sqrtf for float
    R v0 = qdt_4mc / (R)std::sqrt(one + (ux * ux + (uy * uy + uz * uz)));
    R v1 = cbx * cbx + (cby * cby + cbz * cbz);
    R v2 = (v0 * v0) * v1;
    R v3 = v0 * (one + v2 * (one_third + v2 * two_fifteenths));
    R v4 = v3 / (one + v1 * (v3 * v3));
    v4 += v4;
    R t0 = ux + v3 * (uy * cbz - uz * cby);
    R t1 = uy + v3 * (uz * cbx - ux * cbz);
    R t2 = uz + v3 * (ux * cby - uy * cbx);
    ux += v4 * (t1 * cbz - t2 * cby);
    uy += v4 * (t2 * cbx - t0 * cbz);
    uz += v4 * (t0 * cby - t1 * cbx);
    ux += hax; uy += hay; uz += haz;
    P.mem(3, p) = ux; P.mem(4, p) = uy; P.mem(5, p) = uz;
  }
}

// ---------------------------------------------------------------- interpolator
// load_interpolator_array, src/interpolator.cpp:4-124, interior cells only.
template <class R>
void load_interpolator(const R* fields, R* interp, const Grid& g) {
  CellSoA<R, kFieldMembers> F{const_cast<R*>(fields)};
  CellSoA<R, kInterpMembers> I{interp};
  const long ox = 1, oy = g.sx(), oz = g.sx() * g.sy();
  const R fourth = 1.0 / 4.0;
  const R half = 1.0 / 2.0;
  auto four = [&](long i, int m0, R w0, R w1, R w2, R w3) {
    I(i, m0 + 0) = fourth * ((w3 + w0) + (w1 + w2));
    I(i, m0 + 1) = fourth * ((w3 - w0) + (w1 - w2));
    I(i, m0 + 2) = fourth * ((w3 - w0) - (w1 - w2));
    I(i, m0 + 3) = fourth * ((w3 + w0) - (w1 + w2));
  };
#pragma omp parallel for schedule(static)
  for (long z = g.ng; z < g.nz + g.ng; ++z)
    for (long y = g.ng; y < g.ny + g.ng; ++y)
      for (long x = g.ng; x < g.nx + g.ng; ++x) {
        long i = g.vox(x, y, z);
        four(i, EX, F(i, F_EX), F(i + oy, F_EX), F(i + oz, F_EX), F(i + oy + oz, F_EX));
        four(i, EY, F(i, F_EY), F(i + oz, F_EY), F(i + ox, F_EY), F(i + ox + oz, F_EY));
        four(i, EZ, F(i, F_EZ), F(i + ox, F_EZ), F(i + oy, F_EZ), F(i + ox + oy, F_EZ));
        R w0 = F(i, F_CBX), w1 = F(i + ox, F_CBX);
        I(i, CBX) = half * (w1 + w0); I(i, DCBXDX) = half * (w1 - w0);
        w0 = F(i, F_CBY); w1 = F(i + oy, F_CBY);
        I(i, CBY) = half * (w1 + w0); I(i, DCBYDY) = half * (w1 - w0);
        w0 = F(i, F_CBZ); w1 = F(i + oz, F_CBZ);
        I(i, CBZ) = half * (w1 + w0); I(i, DCBZDZ) = half * (w1 - w0);
      }
}

// ---------------------------------------------------------------- accumulator
// unload_accumulator_array, src/accumulator.cpp:45-122, cells [ng, n+ng] per axis.
template <class R>
void unload_accumulator(R* fields, const R* acc, const Grid& g, R dx, R dy, R dz, R dt) {
  CellSoA<R, kFieldMembers> F{fields};
  R cx = 0.25 / (dy * dz * dt);
  R cy = 0.25 / (dz * dx * dt);
  R cz = 0.25 / (dx * dy * dt);
  auto A = [&](long c, int comp, int q) { return acc[(size_t)c * 12 + comp * 4 + q]; };
#pragma omp parallel for schedule(static)
  for (long z = g.ng; z <= g.nz + g.ng; ++z)
    for (long y = g.ng; y <= g.ny + g.ng; ++y)
      for (long x = g.ng; x <= g.nx + g.ng; ++x) {
        long i = g.vox(x, y, z);
        long xd = g.vox(x - 1, y, z), yd = g.vox(x, y - 1, z), zd = g.vox(x, y, z - 1);
        long xzd = g.vox(x - 1, y, z - 1), xyd = g.vox(x - 1, y - 1, z), yzd = g.vox(x, y - 1, z - 1);
        F(i, F_JFX) = cx * (A(i, JX, 0) + A(yd, JX, 1) + A(zd, JX, 2) + A(yzd, JX, 3));
        F(i, F_JFY) = cy * (A(i, JY, 0) + A(zd, JY, 1) + A(xd, JY, 2) + A(xzd, JY, 3));
        F(i, F_JFZ) = cz * (A(i, JZ, 0) + A(xd, JZ, 1) + A(yd, JZ, 2) + A(xyd, JZ, 3));
      }
}

// ---------------------------------------------------------------- ghosts
// Periodic ghost copy of three members, src/fields.h:11-100 (three passes,
// x faces, then y faces, then z faces, in that order).
template <class R>
void ghost_copy(R* fields, const Grid& g, int m0) {
  CellSoA<R, kFieldMembers> F{fields};
  const long nx = g.nx, ny = g.ny, nz = g.nz;
  auto cp = [&](long to, long from) { for (int m = 0; m < 3; ++m) F(to, m0 + m) = F(from, m0 + m); };
  for (long z = 1; z < nz + 1; ++z)
    for (long y = 1; y < ny + 1; ++y) {
      cp(g.vox(nx + 1, y, z), g.vox(1, y, z));
      cp(g.vox(0, y, z), g.vox(nx, y, z));
    }
  for (long x = 0; x < nx + 2; ++x)
    for (long z = 1; z < nz + 1; ++z) {
      cp(g.vox(x, ny + 1, z), g.vox(x, 1, z));
      cp(g.vox(x, 0, z), g.vox(x, ny, z));
    }
  for (long y = 0; y < ny + 2; ++y)
    for (long x = 0; x < nx + 2; ++x) {
      cp(g.vox(x, y, nz + 1), g.vox(x, y, 1));
      cp(g.vox(x, y, 0), g.vox(x, y, nz));
    }
}

// Periodic fold (+=) of the current ghosts, src/fields.h:102-271.
template <class R>
void current_fold(R* fields, const Grid& g) {
  CellSoA<R, kFieldMembers> F{fields};
  const long nx = g.nx, ny = g.ny, nz = g.nz;
  for (long x = 1; x < nx + 1; ++x) {   // jfx: y then z
    for (long z = 1; z <= nz + 1; ++z) F(g.vox(x, 1, z), F_JFX) += F(g.vox(x, ny + 1, z), F_JFX);
    for (long y = 1; y <= ny + 1; ++y) F(g.vox(x, y, 1), F_JFX) += F(g.vox(x, y, nz + 1), F_JFX);
  }
  for (long y = 1; y < ny + 1; ++y) {   // jfy: z then x
    for (long x = 1; x <= nx + 1; ++x) F(g.vox(x, y, 1), F_JFY) += F(g.vox(x, y, nz + 1), F_JFY);
    for (long z = 1; z <= nz + 1; ++z) F(g.vox(1, y, z), F_JFY) += F(g.vox(nx + 1, y, z), F_JFY);
  }
  for (long z = 1; z < nz + 1; ++z) {   // jfz: x then y
    for (long y = 1; y <= ny + 1; ++y) F(g.vox(1, y, z), F_JFZ) += F(g.vox(nx + 1, y, z), F_JFZ);
    for (long x = 1; x <= nx + 1; ++x) F(g.vox(x, 1, z), F_JFZ) += F(g.vox(x, ny + 1, z), F_JFZ);
  }
}

// ---------------------------------------------------------------- EM solver
// EM_Field_Solver::advance_b, src/fields.h:668-719.
template <class R>
void advance_b(R* fields, R px, R py, R pz, const Grid& g) {
  CellSoA<R, kFieldMembers> F{fields};
#pragma omp parallel for schedule(static)
  for (long z = 1; z < g.nz + 1; ++z)
    for (long y = 1; y < g.ny + 1; ++y)
      for (long x = 1; x < g.nx + 1; ++x) {
        long f0 = g.vox(x, y, z), fx = g.vox(x + 1, y, z), fy = g.vox(x, y + 1, z), fz = g.vox(x, y, z + 1);
        F(f0, F_CBX) -= (py * (F(fy, F_EZ) - F(f0, F_EZ)) - pz * (F(fz, F_EY) - F(f0, F_EY)));
        F(f0, F_CBY) -= (pz * (F(fz, F_EX) - F(f0, F_EX)) - px * (F(fx, F_EZ) - F(f0, F_EZ)));
        F(f0, F_CBZ) -= (px * (F(fx, F_EY) - F(f0, F_EY)) - py * (F(fy, F_EX) - F(f0, F_EX)));
      }
  ghost_copy<R>(fields, g, F_CBX);
}

// EM_Field_Solver::advance_e, src/fields.h:618-665.
template <class R>
void advance_e(R* fields, R px, R py, R pz, const Grid& g, R dt_eps0) {
  CellSoA<R, kFieldMembers> F{fields};
  current_fold<R>(fields, g);
  ghost_copy<R>(fields, g, F_JFX);
  const R cj = dt_eps0;
#pragma omp parallel for schedule(static)
  for (long z = 1; z < g.nz + 2; ++z)
    for (long y = 1; y < g.ny + 2; ++y)
      for (long x = 1; x < g.nx + 2; ++x) {
        long f0 = g.vox(x, y, z), fx = g.vox(x - 1, y, z), fy = g.vox(x, y - 1, z), fz = g.vox(x, y, z - 1);
        F(f0, F_EX) = F(f0, F_EX) + (-cj * F(f0, F_JFX)) +
                      (py * (F(f0, F_CBZ) - F(fy, F_CBZ)) - pz * (F(f0, F_CBY) - F(fz, F_CBY)));
        F(f0, F_EY) = F(f0, F_EY) + (-cj * F(f0, F_JFY)) +
                      (pz * (F(f0, F_CBX) - F(fz, F_CBX)) - px * (F(f0, F_CBZ) - F(fx, F_CBZ)));
        F(f0, F_EZ) = F(f0, F_EZ) + (-cj * F(f0, F_JFZ)) +
                      (px * (F(f0, F_CBY) - F(fx, F_CBY)) - py * (F(f0, F_CBX) - F(fy, F_CBX)));
      }
}

// ES solvers, src/fields.h:382-545: (1-D: jf fold first) E -= cj J over every
// cell of the array; e_energy over every cell (ghosts included), double sum.
template <class R>
void es_advance_e(R* fields, const Grid& g, R dt_eps0, bool fold) {
  CellSoA<R, kFieldMembers> F{fields};
  if (fold) current_fold<R>(fields, g);
  const R cj = dt_eps0;
  for (long i = 0; i < g.cells(); ++i) {
    F(i, F_EX) = F(i, F_EX) + (-cj * F(i, F_JFX));
    F(i, F_EY) = F(i, F_EY) + (-cj * F(i, F_JFY));
    F(i, F_EZ) = F(i, F_EZ) + (-cj * F(i, F_JFZ));
  }
}

template <class R>
double es_energy(const R* fields, const Grid& g) {
  CellSoA<R, kFieldMembers> F{const_cast<R*>(fields)};
  double e = 0;
  for (long i = 0; i < g.cells(); ++i) {
    const double a = F(i, F_EX), b = F(i, F_EY), c = F(i, F_EZ);
    e += a * a + b * b + c * c;
  }
  return 0.5 * e;
}

// e_energy / b_energy, src/fields.h:556-615: 0.5 * sum over the interior of
// the squared members, dV = 1.  out[0..1] in real_t accumulation (x fastest),
// out[2..3] the same sums accumulated in double.
template <class R>
void energies(const R* fields, const Grid& g, double out[4]) {
  CellSoA<R, kFieldMembers> F{const_cast<R*>(fields)};
  R se = 0, sb = 0;
  double de = 0, db = 0;
  for (long z = 1; z < g.nz + 1; ++z)
    for (long y = 1; y < g.ny + 1; ++y)
      for (long x = 1; x < g.nx + 1; ++x) {
        long i = g.vox(x, y, z);
        R ex = F(i, F_EX), ey = F(i, F_EY), ez = F(i, F_EZ);
        R bx = F(i, F_CBX), by = F(i, F_CBY), bz = F(i, F_CBZ);
        se += ex * ex + ey * ey + ez * ez;
        sb += bx * bx + by * by + bz * bz;
        de += (double)ex * ex + (double)ey * ey + (double)ez * ez;
        db += (double)bx * bx + (double)by * by + (double)bz * bz;
      }
  const R dV = 1.0;
  out[0] = (double)(R)(se * 0.5f * dV);
  out[1] = (double)(R)(sb * 0.5f * dV);
  out[2] = de * 0.5;
  out[3] = db * 0.5;
}

// ---------------------------------------------------------------- decks
// _Input_Deck::courant_length, src/input/deck.h:191-198.
template <class R>
R courant_length(R lx, R ly, R lz, size_t nx, size_t ny, size_t nz) {
  R w0, w1 = 0;
  if (nx > 1) w0 = nx / lx, w1 += w0 * w0;
  if (ny > 1) w0 = ny / ly, w1 += w0 * w0;
  if (nz > 1) w0 = nz / lz, w1 += w0 * w0;
  return std::sqrt(1 / w1);
}

// Default Particle_Initializer::init, src/input/deck.h:79-158: paired +/- beams
// along x, stratified along y, with a 1e-4 sin perturbation.
template <class R>
void default_particle_init(const Particles<R>& P, size_t n, size_t nx, size_t ny, R dxp,
                           size_t nppc, R w, R v0) {
  for (size_t pi2 = 0; pi2 < n; ++pi2) {
    int sign = -1;
    size_t pi = pi2 / 2;
    if (pi2 % 2 == 0) sign = 1;
    int pic = (int)((2 * pi) % nppc);
    R x = pic * dxp + 0.5 * dxp - 1.0;
    int pre_ghost = (int)(2 * pi / nppc);
    P.mem(0, pi2) = 0.0;
    P.mem(1, pi2) = x;
    P.mem(2, pi2) = 0.0;
    P.mem(6, pi2) = w;
    P.cell(pi2) = (int)(pre_ghost * (nx + 2) + (nx + 2) * (ny + 2) + (nx + 2) + 1);
    R gam = 1.0 / std::sqrt(1.0 - v0 * v0);
    R na = 0.0001 * std::sin(2.0 * 3.1415926 * ((x + 1.0 + pre_ghost * 2) / (2 * ny)));
    P.mem(3, pi2) = sign * v0 * gam * (1.0 + na * sign);
    P.mem(4, pi2) = 0;
    P.mem(5, pi2) = 0;
  }
}

// Parameters of a run, as _Input_Deck holds them after derive_params()
// (src/input/deck.h:254-348) plus the constants main() derives
// (example/example.cpp:77-113,179-181).
// Seeded uniform thermal plasma (the thermal deck's loader, restated from
// cabanapic_gb300/decks.py thermal_particles; no counterpart in the reference,
// whose decks initialise particles on the host: src/input/deck.h:79-158).
// Particle p in interior cell p / ppc (VOXEL order, x fastest) draws from
// Philox4x32-10 (Salmon et al., SC'11) at counters (p, 0) and (p, 1) under
// the 64-bit seed: offsets 2u - 1, momenta Box-Muller normals in double
// rounded once to real_t.  OpenMP over particles; used to make the CPU
// baseline's inputs quickly.
struct U4 { uint32_t x, y, z, w; };

static U4 philox4x32_10(U4 c, uint32_t k0, uint32_t k1) {
  for (int r = 0; r < 10; ++r) {
    const uint64_t p0 = (uint64_t)c.x * 0xD2511F53u, p1 = (uint64_t)c.z * 0xCD9E8D57u;
    c = U4{(uint32_t)(p1 >> 32) ^ c.y ^ k0, (uint32_t)p1, (uint32_t)(p0 >> 32) ^ c.w ^ k1, (uint32_t)p0};
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return c;
}

template <class R>
static R thermal_offset(uint32_t r) {
  if constexpr (sizeof(R) == 4) return (float)(r >> 8) * 0x1p-23f - 1.0f;
  else return (double)r * 0x1p-31 - 1.0;
}

template <class R>
void thermal_particles(const Particles<R>& P, size_t n, long ppc, long nx, long ny, double uth, R weight,
                       uint64_t seed) {
  const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
  const long sx = nx + 2, sy = ny + 2;
  const double pi = 3.14159265358979323846;
#pragma omp parallel for schedule(static)
  for (long p = 0; p < (long)n; ++p) {
    const long k = p / ppc;
    const long ix = k % nx, iy = (k / nx) % ny, iz = k / (nx * ny);
    const U4 a = philox4x32_10(U4{(uint32_t)p, (uint32_t)((uint64_t)p >> 32), 0u, 0u}, k0, k1);
    const U4 b = philox4x32_10(U4{(uint32_t)p, (uint32_t)((uint64_t)p >> 32), 1u, 0u}, k0, k1);
    const double r1 = std::sqrt(-2.0 * std::log(((double)a.w + 1.0) * 0x1p-32));
    const double r2 = std::sqrt(-2.0 * std::log(((double)b.y + 1.0) * 0x1p-32));
    const double t1 = pi * (2.0 * ((double)b.x * 0x1p-32));
    const double t2 = pi * (2.0 * ((double)b.z * 0x1p-32));
    P.mem(0, p) = thermal_offset<R>(a.x);
    P.mem(1, p) = thermal_offset<R>(a.y);
    P.mem(2, p) = thermal_offset<R>(a.z);
    P.mem(3, p) = (R)(uth * (r1 * std::cos(t1)));
    P.mem(4, p) = (R)(uth * (r1 * std::sin(t1)));
    P.mem(5, p) = (R)(uth * (r2 * std::cos(t2)));
    P.mem(6, p) = weight;
    P.cell(p) = (int)((ix + 1) + sx * ((iy + 1) + sy * (iz + 1)));
  }
}

template <class R>
struct Run {
  size_t nx, ny, nz, ng, nppc, num_particles, num_cells;
  int num_steps;
  R dx, dy, dz, dt, c, eps, qsp, me, n0, v0, len_x, len_y, len_z;
  R Npe, Ne, dxp, we, qdt_2mc, cdt_dx, cdt_dy, cdt_dz, dt_eps0, px, py, pz;
};

// The 2stream-em test deck, tests/energy_comparison/2stream-em.cxx:81-114
// (identical to the default deck in src/input/deck.h:432-464).
template <class R>
Run<R> two_stream_em_run() {
  Run<R> r{};
  r.nx = 1; r.ny = 32; r.nz = 1; r.ng = 1; r.nppc = 100; r.num_steps = 6000;
  r.c = 1.0; r.eps = 1.0; r.me = 1.0; r.n0 = 2.0;
  R ec = 1.0;
  r.qsp = -ec;
  r.v0 = 0.0866025403784439;
  R gam = 1.0 / std::sqrt(1.0 - r.v0 * r.v0);
  const R default_grid_len = 1.0;
  r.len_x = default_grid_len;
  // unqualified sqrt(float) in the deck resolves to the C double sqrt(double)
  r.len_y = 0.628318530717959 * (gam * ::sqrt((double)gam));
  r.len_z = default_grid_len;
  r.dt = 0.99 * courant_length<R>(r.len_x, r.len_y, r.len_z, r.nx, r.ny, r.nz) / r.c;
  // derive_params
  r.dx = r.len_x / r.nx; r.dy = r.len_y / r.ny; r.dz = r.len_z / r.nz;
  r.num_cells = (r.nx + 2 * r.ng) * (r.ny + 2 * r.ng) * (r.nz + 2 * r.ng);
  r.num_particles = r.nx * r.ny * r.nz * r.nppc;
  r.Ne = (R)r.num_particles;
  r.Npe = r.n0 * r.len_x * r.len_y * r.len_z;
  // main()
  r.dxp = 2.f / (int)r.nppc;
  r.qdt_2mc = r.qsp * r.dt / (2 * r.me * r.c);
  r.cdt_dx = r.c * r.dt / r.dx; r.cdt_dy = r.c * r.dt / r.dy; r.cdt_dz = r.c * r.dt / r.dz;
  r.dt_eps0 = r.dt / r.eps;
  r.we = (R)r.Npe / (R)r.Ne;
  const R frac = 1.0f;
  r.px = (r.nx > 1) ? frac * r.c * r.dt / r.dx : 0;
  r.py = (r.ny > 1) ? frac * r.c * r.dt / r.dy : 0;
  r.pz = (r.nz > 1) ? frac * r.c * r.dt / r.dz : 0;
  return r;
}

// One time step in the order of example/example.cpp:221-266.
template <class R>
void step(const Particles<R>& P, size_t n, R* fields, R* interp, R* acc, const Grid& g,
          const Run<R>& r, bool literal, long* crossers) {
  load_interpolator<R>(fields, interp, g);
  std::memset(acc, 0, sizeof(R) * 12 * (size_t)g.cells());
  AccSink<R> sink{acc, nullptr, nullptr};
  push_serial<R>(P, n, interp, r.qdt_2mc, r.cdt_dx, r.cdt_dy, r.cdt_dz, r.qsp, sink, g, literal, crossers);
  unload_accumulator<R>(fields, acc, g, r.dx, r.dy, r.dz, r.dt);
  advance_b<R>(fields, R(0.5) * r.px, R(0.5) * r.py, R(0.5) * r.pz, g);
  advance_e<R>(fields, r.px, r.py, r.pz, g, r.dt_eps0);
  advance_b<R>(fields, R(0.5) * r.px, R(0.5) * r.py, R(0.5) * r.pz, g);
}

template <class R>
int run_two_stream_em(int steps, int vl, bool literal, double* out /* steps x 4 */,
                      double* params_out /* 8 */) {
  Run<R> r = two_stream_em_run<R>();
  Grid g{(long)r.nx, (long)r.ny, (long)r.nz, (long)r.ng};
  size_t n = r.num_particles;
  size_t blocks = (n + vl - 1) / vl;
  std::vector<unsigned char> pbuf(blocks * (size_t)vl * (7 * sizeof(R) + sizeof(int)), 0);
  Particles<R> P{pbuf.data(), vl};
  default_particle_init<R>(P, n, r.nx, r.ny, r.dxp, r.nppc, r.we, r.v0);
  size_t cb = (r.num_cells + kCellBlock - 1) / kCellBlock;
  std::vector<R> fields(cb * kCellBlock * kFieldMembers, R(0));
  std::vector<R> interp(cb * kCellBlock * kInterpMembers, R(0));
  std::vector<R> acc(12 * r.num_cells, R(0));
  for (int s = 1; s <= steps; ++s) {
    step<R>(P, n, fields.data(), interp.data(), acc.data(), g, r, literal, nullptr);
    energies<R>(fields.data(), g, out + 4 * (size_t)(s - 1));
  }
  if (params_out) {
    params_out[0] = r.dt; params_out[1] = r.dx; params_out[2] = r.dy; params_out[3] = r.dz;
    params_out[4] = r.qdt_2mc; params_out[5] = r.we; params_out[6] = r.len_y; params_out[7] = r.py;
  }
  return 0;
}

}  // namespace orc

// ================================================================ C interface
// Plain pointers and sizes; loaded with ctypes by the tests and the benchmark.
extern "C" {

struct orc_grid { int64_t nx, ny, nz, ng; };

#define ORC_GRID(gp) orc::Grid g{(long)(gp)->nx, (long)(gp)->ny, (long)(gp)->nz, (long)(gp)->ng}

int orc_push_f32(void* particles, int64_t n, int32_t vl, const float* interp, float qdt_2mc,
                 float cdt_dx, float cdt_dy, float cdt_dz, float qsp, float* acc,
                 float* acc_abs, int32_t* acc_count, const orc_grid* gp, int64_t* crossers) {
  ORC_GRID(gp);
  orc::Particles<float> P{(unsigned char*)particles, vl};
  orc::AccSink<float> sink{acc, acc_abs, acc_count};
  long c = 0;
  orc::push_serial<float>(P, (size_t)n, interp, qdt_2mc, cdt_dx, cdt_dy, cdt_dz, qsp, sink, g, true, &c);
  if (crossers) *crossers = c;
  return 0;
}

int orc_push_f64(void* particles, int64_t n, int32_t vl, const double* interp, double qdt_2mc,
                 double cdt_dx, double cdt_dy, double cdt_dz, double qsp, double* acc,
                 double* acc_abs, int32_t* acc_count, const orc_grid* gp, int32_t literal,
                 int64_t* crossers) {
  ORC_GRID(gp);
  orc::Particles<double> P{(unsigned char*)particles, vl};
  orc::AccSink<double> sink{acc, acc_abs, acc_count};
  long c = 0;
  orc::push_serial<double>(P, (size_t)n, interp, qdt_2mc, cdt_dx, cdt_dy, cdt_dz, qsp, sink, g, literal != 0, &c);
  if (crossers) *crossers = c;
  return 0;
}

// Threaded push (per-thread accumulator copies, then contribute).  Returns
// the number of threads used.
int orc_push_omp_f32(void* particles, int64_t n, int32_t vl, const float* interp, float qdt_2mc,
                     float cdt_dx, float cdt_dy, float cdt_dz, float qsp, float* acc,
                     const orc_grid* gp, int32_t threads) {
  ORC_GRID(gp);
  static std::vector<float> dup;
  orc::Particles<float> P{(unsigned char*)particles, vl};
#ifdef _OPENMP
  if (threads <= 0) threads = omp_get_max_threads();
#else
  threads = 1;
#endif
  orc::push_openmp<float>(P, (size_t)n, interp, qdt_2mc, cdt_dx, cdt_dy, cdt_dz, qsp, acc, g, true, threads, dup);
  return threads;
}

int orc_push_omp_f64(void* particles, int64_t n, int32_t vl, const double* interp, double qdt_2mc,
                     double cdt_dx, double cdt_dy, double cdt_dz, double qsp, double* acc,
                     const orc_grid* gp, int32_t threads) {
  ORC_GRID(gp);
  static std::vector<double> dup;
  orc::Particles<double> P{(unsigned char*)particles, vl};
#ifdef _OPENMP
  if (threads <= 0) threads = omp_get_max_threads();
#else
  threads = 1;
#endif
  orc::push_openmp<double>(P, (size_t)n, interp, qdt_2mc, cdt_dx, cdt_dy, cdt_dz, qsp, acc, g, true, threads, dup);
  return threads;
}

// The threaded FP64 push with sqrt() for gamma (a true FP64 gamma; the
// reference calls sqrtf): the forward map whose finite differences check the
// FP64 adjoint, which differentiates sqrt.  Deterministic for a fixed thread
// count (static schedule, copies summed in thread order).
int orc_push_omp_sqrt_f64(void* particles, int64_t n, int32_t vl, const double* interp, double qdt_2mc,
                          double cdt_dx, double cdt_dy, double cdt_dz, double qsp, double* acc,
                          const orc_grid* gp, int32_t threads) {
  ORC_GRID(gp);
  static std::vector<double> dup;
  orc::Particles<double> P{(unsigned char*)particles, vl};
#ifdef _OPENMP
  if (threads <= 0) threads = omp_get_max_threads();
#else
  threads = 1;
#endif
  orc::push_openmp<double>(P, (size_t)n, interp, qdt_2mc, cdt_dx, cdt_dy, cdt_dz, qsp, acc, g, false, threads, dup);
  return threads;
}

#define ORC_FIELD_FNS(T, SUF)                                                                 \
  int orc_load_interpolator_##SUF(const T* fields, T* interp, const orc_grid* gp) {          \
    ORC_GRID(gp); orc::load_interpolator<T>(fields, interp, g); return 0; }                 \
  int orc_unload_accumulator_##SUF(T* fields, const T* acc, const orc_grid* gp, T dx, T dy,  \
                                   T dz, T dt) {                                             \
    ORC_GRID(gp); orc::unload_accumulator<T>(fields, acc, g, dx, dy, dz, dt); return 0; }   \
  int orc_advance_b_##SUF(T* fields, T px, T py, T pz, const orc_grid* gp) {                 \
    ORC_GRID(gp); orc::advance_b<T>(fields, px, py, pz, g); return 0; }                     \
  int orc_advance_e_##SUF(T* fields, T px, T py, T pz, const orc_grid* gp, T dt_eps0) {      \
    ORC_GRID(gp); orc::advance_e<T>(fields, px, py, pz, g, dt_eps0); return 0; }            \
  int orc_energies_##SUF(const T* fields, const orc_grid* gp, double* out4) {                \
    ORC_GRID(gp); orc::energies<T>(fields, g, out4); return 0; }                            \
  int orc_current_fold_##SUF(T* fields, const orc_grid* gp) {                                \
    ORC_GRID(gp); orc::current_fold<T>(fields, g); return 0; }                              \
  int orc_ghost_copy_##SUF(T* fields, const orc_grid* gp, int32_t first_member) {            \
    ORC_GRID(gp); orc::ghost_copy<T>(fields, g, first_member); return 0; }                  \
  int orc_es_advance_e_##SUF(T* fields, const orc_grid* gp, T dt_eps0, int32_t fold) {       \
    ORC_GRID(gp); orc::es_advance_e<T>(fields, g, dt_eps0, fold != 0); return 0; }          \
  double orc_es_energy_##SUF(const T* fields, const orc_grid* gp) {                          \
    ORC_GRID(gp); return orc::es_energy<T>(fields, g); }

ORC_FIELD_FNS(float, f32)
ORC_FIELD_FNS(double, f64)

int orc_default_particle_init_f32(void* particles, int64_t n, int32_t vl, int64_t nx, int64_t ny,
                                  float dxp, int64_t nppc, float w, float v0) {
  orc::Particles<float> P{(unsigned char*)particles, vl};
  orc::default_particle_init<float>(P, (size_t)n, (size_t)nx, (size_t)ny, dxp, (size_t)nppc, w, v0);
  return 0;
}

int orc_default_particle_init_f64(void* particles, int64_t n, int32_t vl, int64_t nx, int64_t ny,
                                  double dxp, int64_t nppc, double w, double v0) {
  orc::Particles<double> P{(unsigned char*)particles, vl};
  orc::default_particle_init<double>(P, (size_t)n, (size_t)nx, (size_t)ny, dxp, (size_t)nppc, w, v0);
  return 0;
}

// Runs the 2stream-em deck for `steps` steps; out holds steps rows of
// [E_real, B_real, E_double_acc, B_double_acc]; params_out 8 derived values
// [dt, dx, dy, dz, qdt_2mc, we, len_y, py].
int orc_run_two_stream_em(int32_t precision, int32_t steps, int32_t vl, int32_t literal,
                          double* out, double* params_out) {
  if (precision == 4) return orc::run_two_stream_em<float>(steps, vl, literal != 0, out, params_out);
  if (precision == 8) return orc::run_two_stream_em<double>(steps, vl, literal != 0, out, params_out);
  return -1;
}

int orc_uncenter_f32(void* particles, int64_t n, int32_t vl, const float* interp, float qdt_2mc) {
  orc::Particles<float> P{(unsigned char*)particles, vl};
  orc::uncenter<float>(P, (size_t)n, interp, qdt_2mc);
  return 0;
}

int orc_uncenter_f64(void* particles, int64_t n, int32_t vl, const double* interp, double qdt_2mc) {
  orc::Particles<double> P{(unsigned char*)particles, vl};
  orc::uncenter<double>(P, (size_t)n, interp, qdt_2mc);
  return 0;
}

int orc_thermal_particles_f32(void* particles, int64_t n, int32_t vl, int64_t ppc, int64_t nx, int64_t ny,
                              double uth, float weight, uint64_t seed) {
  orc::Particles<float> P{(unsigned char*)particles, vl};
  orc::thermal_particles<float>(P, (size_t)n, (long)ppc, (long)nx, (long)ny, uth, weight, seed);
  return 0;
}

int orc_thermal_particles_f64(void* particles, int64_t n, int32_t vl, int64_t ppc, int64_t nx, int64_t ny,
                              double uth, double weight, uint64_t seed) {
  orc::Particles<double> P{(unsigned char*)particles, vl};
  orc::thermal_particles<double>(P, (size_t)n, (long)ppc, (long)nx, (long)ny, uth, weight, seed);
  return 0;
}

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

}  // extern "C"
