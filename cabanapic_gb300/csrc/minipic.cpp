// minipic.cpp -- the reference's time loop (example/example.cpp:44-290) written
// against the C++ interface in include/cpic/cabana.hpp, running the 2stream-em
// regression deck (tests/energy_comparison/2stream-em.cxx:81-114) on the GPU.
//
// usage: minipic [num_steps] [energies_path]
// Writes `step time E B` per step (dump_energies format).  Built once with
// real_t = float (minipic) and once with REAL_TYPE=double (minipic_f64).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "cpic/cabana.hpp"

namespace {

// _Input_Deck parameters of the 2stream-em deck and derive_params()
// (src/input/deck.h:254-348).
struct Deck {
  size_t nx = 1, ny = 32, nz = 1, num_ghosts = 1, nppc = 100;
  int num_steps = 6000;
  real_t c = 1.0, eps = 1.0, me = 1.0, ec = 1.0, n0 = 2.0;
  real_t qsp = -1.0;
  real_t v0 = 0.0866025403784439;
  real_t len_x = 1.0, len_y = 1.0, len_z = 1.0, dt = 1.0;
  real_t dx, dy, dz, Npe, Ne;
  size_t num_cells, num_particles;

  static real_t courant_length(real_t lx, real_t ly, real_t lz, size_t nx, size_t ny, size_t nz) {
    real_t w0, w1 = 0;
    if (nx > 1) w0 = nx / lx, w1 += w0 * w0;
    if (ny > 1) w0 = ny / ly, w1 += w0 * w0;
    if (nz > 1) w0 = nz / lz, w1 += w0 * w0;
    return ::sqrt(1 / w1);
  }

  Deck() {
    real_t gam = 1.0 / ::sqrt(1.0 - v0 * v0);
    len_y = 0.628318530717959 * (gam * ::sqrt((double)gam));
    dt = 0.99 * courant_length(len_x, len_y, len_z, nx, ny, nz) / c;
    qsp = -ec;
    dx = len_x / nx; dy = len_y / ny; dz = len_z / nz;
    num_cells = (nx + 2 * num_ghosts) * (ny + 2 * num_ghosts) * (nz + 2 * num_ghosts);
    num_particles = nx * ny * nz * nppc;
    Ne = (real_t)num_particles;
    Npe = n0 * len_x * len_y * len_z;
  }
};

// Default Particle_Initializer::init (src/input/deck.h:79-158), on the host,
// packed into the AoSoA layout and copied to the device.
void init_particles(particle_list_t& particles, const Deck& d, real_t dxp, real_t w) {
  const int VL = particle_list_t::vector_length;
  std::vector<unsigned char> h(particles.bytes(), 0);
  const size_t blk = cpic_particle_block_bytes(cpic::kReal, VL);
  auto mem = [&](int m, size_t p) -> real_t& {
    return *reinterpret_cast<real_t*>(h.data() + (p / VL) * blk + ((size_t)m * VL + p % VL) * sizeof(real_t));
  };
  auto cell = [&](size_t p) -> int& {
    return *reinterpret_cast<int*>(h.data() + (p / VL) * blk + (size_t)7 * VL * sizeof(real_t) + (p % VL) * sizeof(int));
  };
  for (size_t pi2 = 0; pi2 < d.num_particles; ++pi2) {
    int sign = (pi2 % 2 == 0) ? 1 : -1;
    size_t pi = pi2 / 2;
    int pic = (int)((2 * pi) % d.nppc);
    real_t x = pic * dxp + 0.5 * dxp - 1.0;
    int pre_ghost = (int)(2 * pi / d.nppc);
    mem(0, pi2) = 0.0;
    mem(1, pi2) = x;
    mem(2, pi2) = 0.0;
    mem(6, pi2) = w;
    cell(pi2) = (int)(pre_ghost * (d.nx + 2) + (d.nx + 2) * (d.ny + 2) + (d.nx + 2) + 1);
    real_t gam = 1.0 / ::sqrt(1.0 - d.v0 * d.v0);
    real_t na = 0.0001 * ::sin(2.0 * 3.1415926 * ((x + 1.0 + pre_ghost * 2) / (2 * d.ny)));
    mem(3, pi2) = sign * d.v0 * gam * (1.0 + na * sign);
    mem(4, pi2) = 0;
    mem(5, pi2) = 0;
  }
  cpic::check_cuda(cudaMemcpy(particles.data(), h.data(), h.size(), cudaMemcpyHostToDevice),
                   "particles upload");
}

}  // namespace

int main(int argc, char** argv) {
  Deck deck;
  const int num_steps = argc > 1 ? std::atoi(argv[1]) : deck.num_steps;
  const char* energies_path = argc > 2 ? argv[2] : "energies.txt";
  // optional per-step particle and field dumps (example.cpp:131-132, 273-277)
  FILE* fptr = argc > 3 ? std::fopen(argv[3], "w") : nullptr;
  FILE* fpfd = argc > 4 ? std::fopen(argv[4], "w") : nullptr;
  try {
    const size_t nx = deck.nx, ny = deck.ny, nz = deck.nz, num_ghosts = deck.num_ghosts;
    const size_t num_cells = deck.num_cells;
    const int npc = (int)deck.nppc;
    real_t dxp = 2.f / (npc);
    const real_t dx = deck.dx, dy = deck.dy, dz = deck.dz;
    real_t dt = deck.dt, c = deck.c;
    real_t qsp = deck.qsp, me = deck.me;
    real_t qdt_2mc = qsp * dt / (2 * me * c);
    real_t cdt_dx = c * dt / dx, cdt_dy = c * dt / dy, cdt_dz = c * dt / dz;
    real_t dt_eps0 = dt / deck.eps;
    real_t frac = 1.0f;
    real_t we = (real_t)deck.Npe / (real_t)deck.Ne;

    particle_list_t particles("particles", deck.num_particles);
    init_particles(particles, deck, dxp, we);
    grid_t* grid = new grid_t();
    interpolator_array_t interpolators("interpolator", num_cells);
    accumulator_array_t accumulators("accumulator", num_cells);
    auto scatter_add = create_scatter_view(accumulators);
    field_array_t fields("fields", num_cells);
    initialize_interpolator(interpolators);
    Field_Solver<EM_Field_Solver> field_solver(fields);
    const Boundary boundary = Periodic;
    const real_t px = (nx > 1) ? frac * c * dt / dx : 0;
    const real_t py = (ny > 1) ? frac * c * dt / dy : 0;
    const real_t pz = (nz > 1) ? frac * c * dt / dz : 0;

    if (fptr) {
      std::fprintf(fptr, "#step=0\n0 ");
      dump_particles(fptr, particles, 0, 0, 0, dx, dy, dz, nx, ny, nz, num_ghosts);
    }
    std::remove(energies_path);  // the reference only truncates at step 0
    for (int step = 1; step <= num_steps; step++) {
      load_interpolator_array(fields, interpolators, nx, ny, nz, num_ghosts);
      clear_accumulator_array(fields, accumulators, nx, ny, nz);
      push(particles, interpolators, qdt_2mc, cdt_dx, cdt_dy, cdt_dz, qsp, scatter_add, grid, nx, ny,
           nz, num_ghosts, boundary);
      contribute(accumulators, scatter_add);
      unload_accumulator_array(fields, accumulators, nx, ny, nz, num_ghosts, dx, dy, dz, dt);
      field_solver.advance_b(fields, real_t(0.5) * px, real_t(0.5) * py, real_t(0.5) * pz, nx, ny, nz, num_ghosts);
      field_solver.advance_e(fields, px, py, pz, nx, ny, nz, num_ghosts, dt_eps0);
      field_solver.advance_b(fields, real_t(0.5) * px, real_t(0.5) * py, real_t(0.5) * pz, nx, ny, nz, num_ghosts);
      dump_energies(field_solver, fields, step, step * dt, px, py, pz, nx, ny, nz, num_ghosts, energies_path);
      if (fpfd) {
        std::fprintf(fpfd, "#step=%d\n", step);
        field_solver.dump_fields(fpfd, fields, 0, 0, 0, dx, dy, dz, nx, ny, nz, num_ghosts);
      }
      if (fptr) {
        std::fprintf(fptr, "#step=%d\n%e ", step, step * dt);
        dump_particles(fptr, particles, 0, 0, 0, dx, dy, dz, nx, ny, nz, num_ghosts);
      }
    }
    if (fptr) std::fclose(fptr);
    if (fpfd) std::fclose(fpfd);
    int32_t st = cpic::read_status();
    delete grid;
    if (st != 0) {
      std::fprintf(stderr, "device status %#x\n", st);
      return 2;
    }
  } catch (const std::exception& e) {
    std::fprintf(stderr, "minipic: %s\n", e.what());
    return 1;
  }
  return 0;
}
