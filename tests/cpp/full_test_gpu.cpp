// The reference's full-step convergence driver (test/full_test.cpp) on the
// GPU through the C++ host mirror include/mifgpu.hpp: Ethier-Steinman exact
// solution on [0,1]x[0,1]x[-1,1], Re = 1e3, final time 1e-4, all Dirichlet.
// Usage: full_test_gpu N Nt [mixed]. Prints the nine error norms of
// test/full_test.cpp:171-175 after adjusting the pressure mean.
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "mifgpu.hpp"

int main(int argc, char **argv) {
  if (argc < 3) {
    std::fprintf(stderr, "usage: %s N Nt [mixed]\n", argv[0]);
    return 2;
  }
  const long N = std::atol(argv[1]);
  const int Nt = std::atoi(argv[2]);
  const bool mixed = argc > 3 && std::strcmp(argv[3], "mixed") == 0;
  mifgpu::Constants c;
  c.n_global = {N, N, N};
  c.size = {1.0, 1.0, 2.0};
  c.origin = {0.0, 0.0, -1.0};
  c.Re = 1e3;
  const double final_time = 1e-4;
  c.dt = final_time / Nt;
  c.precision = mixed ? MIFGPU_MIXED : MIFGPU_FP64;
  c.boundary_kind = MIFGPU_FIELD_ETHIER;
  try {
    mifgpu::Solver solver(c);
    solver.set_exact_velocity(0, 0.0);
    solver.set_exact_pressure(0.0);
    for (int step = 0; step < Nt; ++step) solver.timestep(step * c.dt);  // src/main.cpp:149-156
    solver.adjust_pressure(final_time);
    const auto e = solver.error_norms(final_time);
    std::printf("%.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g\n", e[0], e[1], e[2], e[3], e[4], e[5], e[6],
                e[7], e[8]);
  } catch (const mifgpu::Error &err) {
    std::fprintf(stderr, "%s\n", err.what());
    return 1;
  }
  return 0;
}
