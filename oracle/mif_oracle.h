/*
 * Plain-C restatement of the reference's time step — TEST INFRASTRUCTURE ONLY.
 *
 * This is the oracle the CUDA library is checked against. It restates, on one
 * rank, FattiMei/mpi-incompressible-fluid's projection step
 * (src/Timestep.cpp:97-156), its velocity-only step
 * (src/TimestepVelocity.cpp:60-90), its spectral Poisson solve
 * (src/PressureEquation.cpp:10-274, src/PressureSolverStructures.cpp:5-70),
 * its boundary fill (src/VelocityTensor.cpp:36-233,
 * src/StaggeredTensor.cpp:221-257) and its error norms (src/Norms.cpp:11-118,
 * src/PressureEquation.cpp:288-343), operation for operation, so that built
 * with the same flags it reproduces the reference bit for bit. It is pinned
 * against the reference's own sources in tests/test_oracle.py (when those are
 * present) and against committed fixtures in tests/golden/.
 *
 * Fields use the reference's layout and extents: x fastest,
 * index i + Ex*(j + Ey*k) (include/Tensor.h:137-140,237).
 */
#ifndef MIF_ORACLE_H
#define MIF_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  long n_global[3];  /* include/Constants.h:14-16 convention */
  double size[3];
  double origin[3];
  double Re;
  double dt;
  int periodic[3];
  int exact_kind; /* oracle/manufactured.h MF_* */
} mif_oracle_params;

/* Field ids: 0..2 velocity u,v,w; 3..5 velocity_buffer; 6..8
 * velocity_buffer_2; 9 pressure; 10 pressure_buffer (phi). */
void *mif_oracle_create(const mif_oracle_params *p);
void mif_oracle_destroy(void *h);
int mif_oracle_set_forcing(void *h, int forcing); /* 0 none, 1 velocity forcing, 2 with grad p */
/* Sensitivity probe, not reference behaviour: scales each forcing value by
 * 1 + rel * r with r in [-1, 1) hashed from the point and `seed` (0: off). */
int mif_oracle_set_forcing_noise(void *h, double rel, unsigned seed);
int mif_oracle_extent(void *h, int id, long out[3]);
int mif_oracle_set(void *h, int id, const double *data);
int mif_oracle_get(void *h, int id, double *data);
int mif_oracle_set_exact_velocity(void *h, int set, double t, int include_border);
int mif_oracle_set_exact_pressure(void *h, double t);
int mif_oracle_timestep(void *h, double t_n);
int mif_oracle_timestep_nhn(void *h, double t_n);
int mif_oracle_timestep_velocity(void *h, double t_n);
int mif_oracle_solve_pressure(void *h, int set, double dt);
int mif_oracle_solve_pressure_nhn(void *h, int set, double dt, double t_new, double t_old);
int mif_oracle_apply_bc(void *h, int set, double t);
/* p += phi, then u -= dt grad(phi) on velocity set `set` (interior points):
 * update_pressure + update_velocity_pressure_gradient, src/Timestep.cpp:66-81 */
int mif_oracle_project(void *h, int set, double dt);
int mif_oracle_adjust_pressure(void *h, double t);
int mif_oracle_error_norms(void *h, double t, double out[9]);
double mif_oracle_forcing_value(int kind, int comp, double t, double x, double y, double z, double Re, int with_p);
double mif_oracle_pressure_gradient_value(int kind, int comp, double t, double x, double y, double z, double Re);

#ifdef __cplusplus
}
#endif

#endif
