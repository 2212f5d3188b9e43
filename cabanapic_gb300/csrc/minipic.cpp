// minipic.cpp -- the reference's time loop (example/example.cpp:44-290) written
// against the C++ interface in include/cpic/cabana.hpp, running the 2stream-em
// regression deck (tests/energy_comparison/2stream-em.cxx:81-114) on the GPU.
//
// usage: minipic [num_steps] [energies_path]
// Writes `step time E B` per step (dump_energies format).  Built once with
// real_t = float (minipic) and once with REAL_TYPE=double (minipic_f64).
//
//        minipic thermal N PPC STEPS WARMUP [SORT_INTERVAL]
// The throughput workload through the same C++ interface, end to end: a
// uniform thermal plasma of N^3 cells x PPC particles (dx = 0.05, u_th = 0.05,
// dt = 0.7 Courant, seeded on the device), sorted every SORT_INTERVAL (20)
// steps on the cells SORT_INTERVAL/2 pushes ahead.  After WARMUP steps the timed region (CUDA events) uploads the
// initial particle state from pinned host memory, runs STEPS steps through
// push() and the field solver, reads each step's field energies back to
// pinned host memory and downloads the final particle state; one untimed and
// five timed runs from the same host state.  Prints one JSON line with the
// pushes per second of the median run.
#include <algorithm>
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

// The thermal workload (see the usage above).
int run_thermal(int n, int ppc, int steps, int warmup, int sort_interval) {
  const size_t nx = n, ny = n, nz = n, ng = 1;
  const size_t num_cells = (nx + 2) * (ny + 2) * (nz + 2);
  const size_t np = nx * ny * nz * (size_t)ppc;
  const real_t c = 1, eps = 1, me = 1, n0 = 1, qsp = -1;
  const real_t dx = 0.05, dy = dx, dz = dx, L = (real_t)(n * (double)dx);
  const real_t dt = (real_t)(0.7 * (double)Deck::courant_length(L, L, L, nx, ny, nz) / c);
  const real_t qdt_2mc = qsp * dt / (2 * me * c);
  const real_t cdt_dx = c * dt / dx, cdt_dy = c * dt / dy, cdt_dz = c * dt / dz;
  const real_t dt_eps0 = dt / eps;
  const real_t we = (n0 * L * L * L) / (real_t)np;
  const real_t px = c * dt / dx, py = c * dt / dy, pz = c * dt / dz;
  cudaStream_t s = cpic::current_stream();

  particle_list_t particles("particles", np), spare("sorted", np);
  cpic_grid g = cpic::make_grid(nx, ny, nz, ng);
  cpic::check(cpic_thermal_particles(particles.data(), (int64_t)np, ppc, &g, 0.05, we, 2024, cpic::kReal,
                                     particle_list_t::vector_length, s),
              "cpic_thermal_particles");
  const size_t pbytes = particles.bytes();
  void* h_in = nullptr;
  void* h_out = nullptr;
  double* h_energy = nullptr;
  cpic::check_cuda(cudaHostAlloc(&h_in, pbytes, cudaHostAllocDefault), "cudaHostAlloc");
  cpic::check_cuda(cudaHostAlloc(&h_out, pbytes, cudaHostAllocDefault), "cudaHostAlloc");
  cpic::check_cuda(cudaHostAlloc((void**)&h_energy, sizeof(double) * 2 * (steps + 1), cudaHostAllocDefault),
                   "cudaHostAlloc");
  cpic::check_cuda(cudaMemcpyAsync(h_in, particles.data(), pbytes, cudaMemcpyDeviceToHost, s), "download");

  interpolator_array_t interpolators("interpolator", num_cells);
  accumulator_array_t accumulators("accumulator", num_cells);
  auto scatter_add = create_scatter_view(accumulators);
  field_array_t fields("fields", num_cells);
  initialize_interpolator(interpolators);
  Field_Solver<EM_Field_Solver> field_solver(fields);
  grid_t* grid = new grid_t();
  const size_t sort_bytes = cpic_sort_into_scratch_bytes((int64_t)np, (int64_t)num_cells, cpic::kReal,
                                                         particle_list_t::vector_length);
  cpic::DeviceBytes sort_scratch(sort_bytes), energy_scratch(cpic_energy_scratch_bytes()),
      d_energy(sizeof(double) * 2 * (steps + 1));
  cpic_push_params sort_prm{};
  sort_prm.cdt_dx = cdt_dx; sort_prm.cdt_dy = cdt_dy; sort_prm.cdt_dz = cdt_dz;
  sort_prm.precision = cpic::kReal;
  sort_prm.particle_vl = particle_list_t::vector_length;

  auto step = [&](int k, bool record) {
    load_interpolator_array(fields, interpolators, nx, ny, nz, ng);
    clear_accumulator_array(fields, accumulators, nx, ny, nz);
    if (sort_interval > 0 && k % sort_interval == 0) {
      // keyed by the cells half an interval ahead
      cpic::check(cpic_sort_particles_ahead_into(particles.data(), spare.data(), (int64_t)np, &g, &sort_prm,
                                                 sort_interval / 2, sort_scratch.get(), sort_bytes, s),
                  "cpic_sort_particles_ahead_into");
      particles.swap(spare);
    }
    push(particles, interpolators, qdt_2mc, cdt_dx, cdt_dy, cdt_dz, qsp, scatter_add, grid, nx, ny, nz, ng,
         Periodic);
    contribute(accumulators, scatter_add);
    unload_accumulator_array(fields, accumulators, nx, ny, nz, ng, dx, dy, dz, dt);
    field_solver.advance_b(fields, real_t(0.5) * px, real_t(0.5) * py, real_t(0.5) * pz, nx, ny, nz, ng);
    field_solver.advance_e(fields, px, py, pz, nx, ny, nz, ng, dt_eps0);
    field_solver.advance_b(fields, real_t(0.5) * px, real_t(0.5) * py, real_t(0.5) * pz, nx, ny, nz, ng);
    if (record) {
      double* de = static_cast<double*>(d_energy.get()) + 2 * k;
      cpic::check(cpic_field_energies(fields.data(), &g, cpic::kReal, de, energy_scratch.get(),
                                      energy_scratch.bytes(), s),
                  "cpic_field_energies");
      cpic::check_cuda(cudaMemcpyAsync(h_energy + 2 * k, de, 2 * sizeof(double), cudaMemcpyDeviceToHost, s),
                       "energies");
    }
  };
  for (int k = 0; k < warmup; ++k) step(k, false);
  cpic::check_cuda(cudaStreamSynchronize(s), "warm-up");
  cpic::check(cpic::read_status() == 0 ? CPIC_OK : CPIC_ECUDA, "device status after warm-up");
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  // one untimed pass, then five timed runs from the same host state; the
  // median is reported (the host link is shared with the rest of the machine)
  constexpr int kRuns = 5;
  float runs[kRuns + 1];
  for (int r = 0; r <= kRuns; ++r) {
    cudaEventRecord(e0, s);
    cpic::check_cuda(cudaMemcpyAsync(particles.data(), h_in, pbytes, cudaMemcpyHostToDevice, s), "upload");
    cpic::check_cuda(cudaMemsetAsync(fields.data(), 0, fields.bytes(), s), "fields reset");
    for (int k = 0; k < steps; ++k) step(k, true);
    cpic::check_cuda(cudaMemcpyAsync(h_out, particles.data(), pbytes, cudaMemcpyDeviceToHost, s), "download");
    cudaEventRecord(e1, s);
    cpic::check_cuda(cudaEventSynchronize(e1), "timed region");
    cudaEventElapsedTime(&runs[r], e0, e1);
  }
  float sorted_runs[kRuns];
  std::copy(runs + 1, runs + kRuns + 1, sorted_runs);
  std::sort(sorted_runs, sorted_runs + kRuns);
  const float ms = sorted_runs[kRuns / 2];
  const int32_t st = cpic::read_status();
  std::printf("{\"path\": \"C++ push() interface (include/cpic/cabana.hpp)\", \"particles\": %zu, "
              "\"steps\": %d, \"warmup\": %d, \"ms\": %.4f, \"runs_ms\": [%.3f, %.3f, %.3f, %.3f, %.3f], "
              "\"pushes_per_s\": %.6e, "
              "\"h2d_bytes\": %zu, \"d2h_bytes\": %zu, \"energy_last\": [%.9e, %.9e], \"status\": %d}\n",
              np, steps, warmup, ms, runs[1], runs[2], runs[3], runs[4], runs[5], (double)np * steps / (ms * 1e-3),
              pbytes,
              pbytes + sizeof(double) * 2 * (size_t)steps, h_energy[2 * (steps - 1)],
              h_energy[2 * (steps - 1) + 1], st);
  cudaFreeHost(h_in);
  cudaFreeHost(h_out);
  cudaFreeHost(h_energy);
  delete grid;
  return st == 0 ? 0 : 2;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc > 1 && std::strcmp(argv[1], "thermal") == 0) {
    if (argc < 6) {
      std::fprintf(stderr, "usage: minipic thermal N PPC STEPS WARMUP [SORT_INTERVAL]\n");
      return 1;
    }
    try {
      return run_thermal(std::atoi(argv[2]), std::atoi(argv[3]), std::atoi(argv[4]), std::atoi(argv[5]),
                         argc > 6 ? std::atoi(argv[6]) : 20);
    } catch (const std::exception& e) {
      std::fprintf(stderr, "minipic: %s\n", e.what());
      return 1;
    }
  }
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
