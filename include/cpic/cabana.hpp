// cabana.hpp -- the reference's C++ hot-path interface over the C ABI.
//
// Drop-in surface for code written against CabanaPIC's headers: the same
// type names (particle_list_t, interpolator_array_t, accumulator_array_t,
// field_array_t, Boundary), the same free functions (push, load_interpolator_array,
// initialize_interpolator, clear_accumulator_array, unload_accumulator_array)
// and the same Field_Solver<EM_Field_Solver> methods, with the reference's
// argument lists.  real_t is chosen with REAL_TYPE exactly as in src/types.h.
//
// The containers here own device memory with the reference's byte layouts
// (layout.h).  A Kokkos/Cabana build would instead pass its own views'
// .data() pointers to the cpic_* functions directly, from the bodies of its
// push() and field functions.
// Errors: a non-zero C-ABI return code throws cpic::Error.
#pragma once

#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <functional>
#include <stdexcept>
#include <utility>
#include <string>
#include <vector>

#include "capi.h"

#ifndef REAL_TYPE
typedef float real_t;
#else
typedef REAL_TYPE real_t;
#endif

#ifndef CPIC_PARTICLE_VL
#define CPIC_PARTICLE_VL 32  // Cabana's default vector length for CUDA memory
#endif

namespace cpic {

struct Error : std::runtime_error {
  int code;
  Error(const std::string& what, int c) : std::runtime_error(what + ": " + cpic_strerror(c)), code(c) {}
};

inline void check(int rc, const char* what) {
  if (rc != CPIC_OK) throw Error(what, rc);
}
inline void check_cuda(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

constexpr int kReal = (int)sizeof(real_t);

// Device buffer with the lifetime of the owning container.
class DeviceBytes {
 public:
  DeviceBytes() = default;
  explicit DeviceBytes(size_t n) : n_(n) {
    if (n) {
      check_cuda(cudaMalloc(&p_, n), "cudaMalloc");
      check_cuda(cudaMemset(p_, 0, n), "cudaMemset");
    }
  }
  DeviceBytes(const DeviceBytes&) = delete;
  DeviceBytes& operator=(const DeviceBytes&) = delete;
  DeviceBytes(DeviceBytes&& o) noexcept : p_(o.p_), n_(o.n_) { o.p_ = nullptr; o.n_ = 0; }
  ~DeviceBytes() { if (p_) cudaFree(p_); }
  void* get() const { return p_; }
  size_t bytes() const { return n_; }
  void swap(DeviceBytes& o) noexcept {
    std::swap(p_, o.p_);
    std::swap(n_, o.n_);
  }

 private:
  void* p_ = nullptr;
  size_t n_ = 0;
};

}  // namespace cpic

// Boundary, src/input/deck.h:9-12
enum Boundary { Reflect = CPIC_REFLECT, Periodic = CPIC_PERIODIC };

// grid_t is unused by push (src/move_p.h:68); an opaque stand-in.
struct grid_t {};

// particle_list_t: Cabana::AoSoA<MemberTypes<real_t x7, int>, MemorySpace>
class particle_list_t {
 public:
  static constexpr int vector_length = CPIC_PARTICLE_VL;
  particle_list_t(const char* /*label*/, size_t n)
      : n_(n), mem_(cpic_particle_list_bytes((int64_t)n, cpic::kReal, vector_length)) {}
  size_t size() const { return n_; }
  void* data() const { return mem_.get(); }
  size_t bytes() const { return mem_.bytes(); }
  // exchanges the storage of two lists of the same size (a double-buffered
  // sort writes the sorted list into the second one)
  void swap(particle_list_t& o) noexcept {
    std::swap(n_, o.n_);
    mem_.swap(o.mem_);
  }

 private:
  size_t n_;
  cpic::DeviceBytes mem_;
};

template <int NM>
class cell_aosoa_t {
 public:
  cell_aosoa_t(const char* /*label*/, size_t num_cells)
      : n_(num_cells), mem_(cpic_cell_array_bytes((int64_t)num_cells, NM, cpic::kReal)) {}
  size_t size() const { return n_; }
  void* data() const { return mem_.get(); }
  size_t bytes() const { return mem_.bytes(); }

 private:
  size_t n_;
  cpic::DeviceBytes mem_;
};

// interpolator_array_t / field_array_t: AoSoA with 32-cell blocks
typedef cell_aosoa_t<CPIC_INTERP_MEMBERS> interpolator_array_t;
typedef cell_aosoa_t<CPIC_FIELD_MEMBERS> field_array_t;

// accumulator_array_t: Kokkos::View<real_t*[3][4]>, LayoutRight (the
// reference's host build) unless CPIC_ACCUMULATOR_LAYOUT_LEFT is defined: then
// Kokkos' LayoutLeft, the layout the same View has in a Kokkos-Cuda build
// (src/types.h:120); push and unload_accumulator_array follow.
class accumulator_array_t {
 public:
#ifdef CPIC_ACCUMULATOR_LAYOUT_LEFT
  static constexpr bool layout_left = true;
#else
  static constexpr bool layout_left = false;
#endif
  accumulator_array_t(const char* /*label*/, size_t num_cells)
      : n_(num_cells), mem_(num_cells * CPIC_ACC_VALUES * sizeof(real_t)) {}
  size_t extent(int) const { return n_; }
  size_t size() const { return n_; }
  void* data() const { return mem_.get(); }

 private:
  size_t n_;
  cpic::DeviceBytes mem_;
};

// The reference scatters through a Kokkos ScatterView (example.cpp:139) and
// then calls contribute()/reset_except().  The device kernels add straight
// into the accumulator, so the scatter view is a thin handle and contribute is
// a no-op.
struct accumulator_scatter_t {
  accumulator_array_t* target;
  void* data() const { return target->data(); }
};
inline accumulator_scatter_t create_scatter_view(accumulator_array_t& a) { return {&a}; }
inline void contribute(accumulator_array_t&, accumulator_scatter_t&) {}

namespace cpic {

// Stream used by the C++ interface (0 = legacy default stream, like Kokkos' default instance).
inline cpic_stream_t& current_stream() {
  static cpic_stream_t s = nullptr;
  return s;
}

// Device status word shared by the push calls.
inline int32_t* status_word() {
  static int32_t* w = nullptr;
  if (!w) {
    check_cuda(cudaMalloc(&w, sizeof(int32_t)), "cudaMalloc(status)");
    check_cuda(cudaMemset(w, 0, sizeof(int32_t)), "cudaMemset(status)");
  }
  return w;
}

inline cpic_grid make_grid(size_t nx, size_t ny, size_t nz, size_t ng, Boundary b = Periodic) {
  cpic_grid g;
  g.nx = (int64_t)nx; g.ny = (int64_t)ny; g.nz = (int64_t)nz; g.num_ghosts = (int64_t)ng;
  g.boundary = (int32_t)b; g.reserved = 0;
  return g;
}

// Boundary of the field solver: a global of the deck in the reference.
inline Boundary& field_boundary() {
  static Boundary b = Periodic;
  return b;
}

inline int32_t read_status(bool clear = true) {
  int32_t h = 0;
  check(cpic_status_read(status_word(), current_stream(), &h), "cpic_status_read");
  if (clear) check(cpic_status_clear(status_word(), current_stream()), "cpic_status_clear");
  return h;
}

inline void* acc_ptr(accumulator_array_t& a) { return a.data(); }
inline void* acc_ptr(accumulator_scatter_t& a) { return a.data(); }

}  // namespace cpic

// push(), src/push.h:7-23 -- same parameter list.
template <class _accumulator>
void push(particle_list_t& particles, interpolator_array_t& f0, real_t qdt_2mc, real_t cdt_dx,
          real_t cdt_dy, real_t cdt_dz, real_t qsp, _accumulator& a0, grid_t* /*g*/,
          const size_t nx, const size_t ny, const size_t nz, const size_t num_ghosts,
          Boundary boundary) {
  cpic_grid grid = cpic::make_grid(nx, ny, nz, num_ghosts, boundary);
  cpic_push_params prm;
  prm.qdt_2mc = qdt_2mc; prm.cdt_dx = cdt_dx; prm.cdt_dy = cdt_dy; prm.cdt_dz = cdt_dz;
  prm.qsp = qsp; prm.precision = cpic::kReal; prm.particle_vl = particle_list_t::vector_length;
  prm.flags = accumulator_array_t::layout_left ? CPIC_PUSH_ACC_LAYOUT_LEFT : 0; prm.reserved = 0;
  cpic::check(cpic_push(particles.data(), (int64_t)particles.size(), f0.data(), cpic::acc_ptr(a0),
                        &grid, &prm, cpic::status_word(), cpic::current_stream()),
              "push");
}

// load_interpolator_array, src/interpolator.h:14-21 (views by value)
inline void load_interpolator_array(field_array_t& fields, interpolator_array_t& interpolators,
                                    size_t nx, size_t ny, size_t nz, size_t ng) {
  cpic_grid g = cpic::make_grid(nx, ny, nz, ng, cpic::field_boundary());
  cpic::check(cpic_load_interpolator(fields.data(), interpolators.data(), &g, cpic::kReal,
                                     cpic::current_stream()),
              "load_interpolator_array");
}

// initialize_interpolator, src/interpolator.h:23
inline void initialize_interpolator(interpolator_array_t& f0) {
  cpic::check(cpic_initialize_interpolator(f0.data(), (int64_t)f0.size(), cpic::kReal,
                                           cpic::current_stream()),
              "initialize_interpolator");
}

// clear_accumulator_array, src/accumulator.h:15-21
inline void clear_accumulator_array(field_array_t& /*fields*/, accumulator_array_t& accumulators,
                                    size_t /*nx*/, size_t /*ny*/, size_t /*nz*/) {
  cpic::check(cpic_clear_accumulator(accumulators.data(), (int64_t)accumulators.size(), cpic::kReal,
                                     cpic::current_stream()),
              "clear_accumulator_array");
}

// unload_accumulator_array, src/accumulator.h:23-32
inline void unload_accumulator_array(field_array_t& fields, accumulator_array_t& accumulators,
                                     size_t nx, size_t ny, size_t nz, size_t ng, real_t dx,
                                     real_t dy, real_t dz, real_t dt) {
  cpic_grid g = cpic::make_grid(nx, ny, nz, ng, cpic::field_boundary());
  auto unload = accumulator_array_t::layout_left ? cpic_unload_accumulator_left : cpic_unload_accumulator;
  cpic::check(unload(fields.data(), accumulators.data(), &g, dx, dy, dz, dt, cpic::kReal, cpic::current_stream()),
              "unload_accumulator_array");
}

// EM_Field_Solver, src/fields.h:550-720 (energies accumulated in double)
class EM_Field_Solver {
 public:
  void advance_b(field_array_t& fields, real_t px, real_t py, real_t pz, size_t nx, size_t ny,
                 size_t nz, size_t ng) {
    cpic_grid g = cpic::make_grid(nx, ny, nz, ng, cpic::field_boundary());
    cpic::check(cpic_advance_b(fields.data(), px, py, pz, &g, cpic::kReal, cpic::current_stream()),
                "advance_b");
  }
  void advance_e(field_array_t& fields, real_t px, real_t py, real_t pz, size_t nx, size_t ny,
                 size_t nz, size_t ng, real_t dt_eps0) {
    cpic_grid g = cpic::make_grid(nx, ny, nz, ng, cpic::field_boundary());
    cpic::check(cpic_advance_e(fields.data(), px, py, pz, &g, dt_eps0, cpic::kReal,
                               cpic::current_stream()),
                "advance_e");
  }
  double e_energy(field_array_t& fields, real_t, real_t, real_t, size_t nx, size_t ny, size_t nz,
                  size_t ng) {
    return energies(fields, nx, ny, nz, ng)[0];
  }
  double b_energy(field_array_t& fields, real_t, real_t, real_t, size_t nx, size_t ny, size_t nz,
                  size_t ng) {
    return energies(fields, nx, ny, nz, ng)[1];
  }

 private:
  cpic::DeviceBytes out_{2 * sizeof(double)};
  cpic::DeviceBytes scratch_{cpic_energy_scratch_bytes()};
  std::vector<double> energies(field_array_t& fields, size_t nx, size_t ny, size_t nz, size_t ng) {
    cpic_grid g = cpic::make_grid(nx, ny, nz, ng, cpic::field_boundary());
    cpic::check(cpic_field_energies(fields.data(), &g, cpic::kReal, static_cast<double*>(out_.get()),
                                    scratch_.get(), scratch_.bytes(), cpic::current_stream()),
                "field energies");
    std::vector<double> h(2);
    cpic::check_cuda(cudaMemcpyAsync(h.data(), out_.get(), 2 * sizeof(double), cudaMemcpyDeviceToHost,
                                     reinterpret_cast<cudaStream_t>(cpic::current_stream())),
                     "energies copy");
    cpic::check_cuda(cudaStreamSynchronize(reinterpret_cast<cudaStream_t>(cpic::current_stream())),
                     "energies sync");
    return h;
  }
};

namespace cpic {
// Device-computed dump values copied to the host (the reference deep-copies
// the whole array first; only 2 reals per particle or x cell cross here).
inline std::vector<real_t> dump_values(size_t n2, const char* what,
                                       const std::function<int(void*)>& fill) {
  DeviceBytes d(n2 * sizeof(real_t));
  check(fill(d.get()), what);
  std::vector<real_t> h(n2);
  cudaStream_t s = reinterpret_cast<cudaStream_t>(current_stream());
  check_cuda(cudaMemcpyAsync(h.data(), d.get(), n2 * sizeof(real_t), cudaMemcpyDeviceToHost, s), what);
  check_cuda(cudaStreamSynchronize(s), what);
  return h;
}
}  // namespace cpic

// Field_Solver<Solver_Type>, src/fields.h:274-379: zeroes the fields on construction.
template <class Solver_Type>
class Field_Solver : public Solver_Type {
 public:
  explicit Field_Solver(field_array_t& fields) { init(fields); }
  void init(field_array_t& fields) {
    cpic::check_cuda(cudaMemsetAsync(fields.data(), 0, fields.bytes(),
                                     reinterpret_cast<cudaStream_t>(cpic::current_stream())),
                     "init_fields");
  }
  // dump_fields, src/fields.h:318-350: x and ex along the first x row.
  void dump_fields(FILE* fp, field_array_t& fields, real_t xmin, real_t, real_t, real_t dx, real_t,
                   real_t, size_t nx, size_t ny, size_t nz, size_t ng) {
    cpic_grid g = cpic::make_grid(nx, ny, nz, ng, cpic::field_boundary());
    std::vector<real_t> v = cpic::dump_values(2 * nx, "dump_fields", [&](void* d) {
      return cpic_field_dump_values(fields.data(), &g, cpic::kReal, xmin, dx, d, cpic::current_stream());
    });
    for (size_t i = 0; i < nx; ++i) fprintf(fp, "%e %e\n", v[2 * i], v[2 * i + 1]);
    fprintf(fp, "\n\n");
  }
};

// dump_particles, src/helpers.h:31-61: x position and ux of every particle.
inline void dump_particles(FILE* fp, const particle_list_t& particles, const real_t xmin, const real_t,
                           const real_t, const real_t dx, const real_t, const real_t, size_t nx,
                           size_t ny, size_t nz, size_t ng) {
  cpic_grid g = cpic::make_grid(nx, ny, nz, ng, Periodic);
  const size_t n = particles.size();
  std::vector<real_t> v = cpic::dump_values(2 * n, "dump_particles", [&](void* d) {
    return cpic_particle_dump_values(particles.data(), (int64_t)n, particle_list_t::vector_length, &g,
                                     cpic::kReal, xmin, dx, d, cpic::current_stream());
  });
  for (size_t i = 0; i < n; ++i) fprintf(fp, "%e  %e ", v[2 * i], v[2 * i + 1]);
  fprintf(fp, "\n");
}

// dump_energies, src/fields.h:722-763: appends `step time E B` to energies.txt
// (truncating at step 0), std::ostream default formatting, and prints the same
// line to stdout as printf("%d %f %e %e\n") does there.
#include <fstream>
template <typename field_solver_t>
void dump_energies(field_solver_t& field_solver, field_array_t& fields, int step, real_t time,
                   real_t px, real_t py, real_t pz, size_t nx, size_t ny, size_t nz, size_t ng,
                   const char* path = "energies.txt") {
  double e_en = field_solver.e_energy(fields, px, py, pz, nx, ny, nz, ng);
  double b_en = field_solver.b_energy(fields, px, py, pz, nx, ny, nz, ng);
  std::ofstream f;
  if (step == 0) f.open(path, std::ofstream::out | std::ofstream::trunc);
  else f.open(path, std::ios::app);
  f << step << " " << time << " " << e_en << " " << b_en << std::endl;
  printf("%d %f %e %e\n", step, (double)time, e_en, b_en);
}
