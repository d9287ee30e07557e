"""Cases of the golden fixtures (shared by make_golden.py and the tests).

Each case is small enough for the oracle to finish in milliseconds. Shapes
are ragged on purpose (no two axes equal, odd and even point counts) and
cover every boundary combination the reference supports on one rank.
"""
TWO_PI = 6.283185307179586
HALF_PI = 1.5707963267948966

CASES = {
    # test/full_test.cpp set-up: Ethier-Steinman exact solution, all Dirichlet.
    "full_dirichlet_ethier": dict(
        case=dict(n_global=(9, 10, 11), size=(1.0, 1.0, 2.0), origin=(0.0, 0.0, -1.0), Re=1e3, dt=1e-4,
                  exact_kind=2), init="exact", op="timestep", steps=3),
    # BASELINE config-1 velocity family (SINCOS), reference semantics (no forcing).
    "full_dirichlet_sincos": dict(
        case=dict(n_global=(8, 9, 7), size=(1.0, 1.0, 1.0), Re=1e3, dt=1e-3, exact_kind=1),
        init="exact", t0=0.5, op="timestep", steps=2),
    # Periodic box, seeded random fields (BASELINE configs 2 and 4 shape).
    "full_periodic_random": dict(
        case=dict(n_global=(9, 8, 10), size=(TWO_PI, TWO_PI, TWO_PI), Re=1600.0, dt=2e-3,
                  periodic=(True, True, True)), init="random", seed=7, op="timestep", steps=2),
    # Channel: periodic x and z, Dirichlet (no-slip) y (BASELINE config 3 shape).
    "full_channel_random": dict(
        case=dict(n_global=(9, 7, 8), size=(4 * 3.141592653589793, 2.0, TWO_PI), Re=5000.0, dt=5e-4,
                  periodic=(True, False, True)), init="random", seed=11, op="timestep", steps=2),
    # Periodic y only.
    "full_periodic_y": dict(
        case=dict(n_global=(7, 9, 8), size=(1.0, TWO_PI, 1.5), Re=500.0, dt=1e-3, periodic=(False, True, False),
                  exact_kind=2), init="exact", op="timestep", steps=2),
    # Non-homogeneous Neumann variant (src/Timestep.cpp:143-149).
    "full_nhn_ethier": dict(
        case=dict(n_global=(8, 9, 10), size=(1.0, 1.0, 2.0), origin=(0.0, 0.0, -1.0), Re=1e3, dt=1e-4,
                  exact_kind=2), init="exact", op="timestep_nhn", steps=2),
    # Velocity-only step with forcing (src/TimestepVelocity.cpp:60-90).
    "velocity_sincos": dict(
        case=dict(n_global=(9, 8, 10), size=(1.0, 1.0, 1.0), Re=1e4, dt=1e-4, exact_kind=1),
        init="exact", t0=0.25, op="timestep_velocity", steps=3),
    # Stand-alone Poisson solves (test/pressure_test_hn.cpp / _mixed.cpp shapes N x 3N x 5N).
    "poisson_neumann": dict(
        case=dict(n_global=(4, 12, 20), size=(TWO_PI, TWO_PI, TWO_PI), Re=1.0, dt=1.0),
        init="random", seed=3, op="solve_pressure", solve_dt=1.0),
    "poisson_mixed": dict(
        case=dict(n_global=(5, 15, 25), size=(TWO_PI, TWO_PI, TWO_PI), Re=1.0, dt=1.0, periodic=(False, False, True)),
        init="random", seed=5, op="solve_pressure", solve_dt=1.0),
    "poisson_periodic_odd": dict(
        case=dict(n_global=(8, 10, 12), size=(TWO_PI, TWO_PI, TWO_PI), Re=1.0, dt=1.0, periodic=(True, True, True)),
        init="random", seed=9, op="solve_pressure", solve_dt=0.5),
    # Stand-alone non-homogeneous Neumann solve on the test/pressure_test_nhn.cpp
    # shape (N x 3N x 5N on [-pi/2, 0]^3, dt = 1): random velocity, boundary
    # data = grad p(t_old) - grad p(t_new) of the Ethier-Steinman pressure.
    "poisson_nhn": dict(
        case=dict(n_global=(4, 12, 20), size=(HALF_PI, HALF_PI, HALF_PI), origin=(-HALF_PI, -HALF_PI, -HALF_PI),
                  Re=1.0, dt=1.0, exact_kind=2),
        init="random", seed=21, op="solve_pressure_nhn", solve_dt=1.0, t_new=0.3, t_old=0.2),
    # Boundary fill alone.
    "bc_ethier": dict(
        case=dict(n_global=(6, 7, 8), size=(1.0, 1.0, 2.0), origin=(0.0, 0.0, -1.0), Re=1e3, dt=1e-4,
                  exact_kind=2), init="random", seed=13, op="apply_bc", bc_t=0.3),
}
