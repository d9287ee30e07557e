// Calls every method of the C++ mirror (include/mifgpu.hpp) once, so that a
// compile and a link with no undefined symbol show that the mirror covers
// the whole C ABI with matching signatures. It is built by
// tests/test_abi.py and never run.
#include <array>
#include <vector>

#include "mifgpu.hpp"

int main() {
  mifgpu::Constants c;
  c.n_global = {9, 9, 9};
  mifgpu::Solver s(c);
  std::vector<double> buf(16 * 16 * 16);
  double *b = buf.data();
  s.extent(mifgpu::U);
  s.upload(mifgpu::U, b);
  s.download(mifgpu::P, b);
  s.timestep(b, b, b, 0.0, b);
  s.timestep(0.0);
  s.run(0.0, 1);
  s.timestep_nhn(0.0);
  s.timestep_velocity(0.0);
  s.run_velocity(0.0, 2);
  s.solve_pressure_equation_homogeneous_periodic(0, 1.0);
  s.apply_bc(0, 0.0);
  s.set_boundary_values(1, b, b, b);
  s.set_pressure_gradient_faces(1, {b, b, b, b, b, b});
  s.solve_pressure_equation_non_homogeneous_neumann(0, 1.0, {b, b, b, b, b, b});
  s.adjust_pressure(0.0);
  s.error_norms(0.0);
  s.set_exact_velocity(0, 0.0);
  s.set_exact_pressure(0.0);
  s.calculate_velocity_divergence(0, 1.0);
  s.update_pressure_and_velocity(0, 1.0);
  s.writeVTK("a.vtk");
  s.writeDat("a.dat", 0, 0.5, 0.5, 0.5);
  s.writeVTKFullMesh("b.vtk");
  s.set_stream(nullptr);
  s.synchronize();
  double loss = 0.0;
  std::array<double, 3> ms{};
  s.gradient_ke(0.0, 2, 1, {0.0, 1.0, 0.0, 1.0, 0.0, 1.0}, &loss, &ms);
  s.backward(0.0, 2, 1, b, b, b, b, &ms);
  s.download_adjoint(mifgpu::U, b);
  s.set_forcing_amplitude(1.0);
  s.velocity_error_norms_noalloc(0.0);
  s.profile_step(0.0, 1);
  s.launch_count();
  s.device_bytes();
  mifgpu::Solver::probe_fp64_fma();
  s.handle();
  return 0;
}
