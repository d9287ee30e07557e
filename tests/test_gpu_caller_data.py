"""Caller-supplied boundary data (boundary_kind MIFGPU_FIELD_CALLER), through
the C ABI.

The reference's step takes its wall data from the caller's exact_velocity
and exact_pressure_gradient functions (include/Timestep.h:16-27). With
MIFGPU_FIELD_CALLER the library takes, per stage, the face values that
VelocityTensor::apply_bc writes (src/VelocityTensor.cpp:36-233) and the
normal pressure-gradient data of the non-homogeneous Neumann step. Here the
caller is the oracle itself: its own apply_bc (bit-identical to the
reference's) fills a scratch velocity set at each stage time, and its
analytic gradient gives the Neumann data, so the caller path must reproduce
the compiled-in family path and the oracle's step within 1e-12.
"""
import numpy as np
import pytest

from test_gpu_parity import FP64_TOL, field_err, make_solver, rel_err

pytestmark = pytest.mark.gpu


def stage_times(t_n, dt):
    """src/Timestep.cpp:97-104, in the same double operations."""
    dt_1 = 64.0 / 120.0 * dt
    time_1 = t_n + dt_1
    dt_2 = 16.0 / 120.0 * dt
    time_2 = time_1 + dt_2
    return (time_1, time_2, t_n + dt)


def feed_stage_data(O, scratch, g, t_n, dt, nhn=False):
    """What a reference-side binding does before each step: the caller's
    boundary values at the three stage times (apply_bc on a scratch set) and,
    for the nhn step, the gradient differences over each stage."""
    times = stage_times(t_n, dt)
    for k, tk in enumerate(times):
        scratch.apply_bc(0, tk)
        g.set_boundary_values(1 + k, *(scratch.get(n) for n in ("u", "v", "w")))
    if nhn:
        prev = (t_n,) + times[:2]
        for k in range(3):
            g.set_pressure_gradient_faces(1 + k, O.gradient_faces(scratch.case, times[k], prev[k]))


@pytest.mark.parametrize("shape,periodic,kind", [
    ((17, 18, 19), (False, False, False), 2),
    ((18, 17, 16), (False, True, False), 2),
    ((16, 17, 18), (True, False, True), 1),
])
def test_caller_boundary_matches_family_and_oracle(oracle_lib, mifgpu_lib, cuda_device, shape, periodic, kind):
    O, mg = oracle_lib, mifgpu_lib
    kw = dict(n_global=shape, size=(1.0, 1.1, 1.2), origin=(0.0, -0.5, 0.2), Re=700.0, dt=2e-4, periodic=periodic,
              exact_kind=kind)
    case = O.Case(**kw)
    o = O.OracleSolver(case)
    o.set_exact_velocity(0, 0.1, True)
    o.set_exact_pressure(0.1)
    st = {n: o.get(n) for n in ("u", "v", "w", "p")}
    fam = make_solver(mg, kw)
    call = make_solver(mg, dict(kw, exact_kind=mg.FIELD_CALLER))
    fam.load_state(st)
    call.load_state(st)
    scratch = O.OracleSolver(case)
    for k in range(3):
        t = 0.1 + k * kw["dt"]
        feed_stage_data(O, scratch, call, t, kw["dt"])
        call.timestep(t)
        fam.timestep(t)
        o.timestep(t)
    want = {n: o.get(n) for n in O.FIELD_NAMES}
    for n in O.FIELD_NAMES:
        assert field_err(n, call.download(n), want[n], want["p"]) <= FP64_TOL, n
        assert field_err(n, call.download(n), fam.download(n), want["p"]) <= FP64_TOL, n
    # the drop-in host call takes the same data
    host = [np.ascontiguousarray(want[n]) for n in ("u", "v", "w", "p")]
    t = 0.1 + 3 * kw["dt"]
    feed_stage_data(O, scratch, call, t, kw["dt"])
    call.timestep_host(t, *host)
    o.timestep(t)
    for n, a in zip(("u", "v", "w", "p"), host):
        assert rel_err(a, o.get(n)) <= FP64_TOL, n
    fam.close()
    call.close()


def test_caller_nhn_step_matches_oracle(oracle_lib, mifgpu_lib, cuda_device):
    """The non-homogeneous Neumann step with both kinds of caller data."""
    O, mg = oracle_lib, mifgpu_lib
    kw = dict(n_global=(13, 14, 15), size=(1.0, 1.0, 2.0), origin=(0.0, 0.0, -1.0), Re=1e3, dt=1e-4, exact_kind=2)
    case = O.Case(**kw)
    o = O.OracleSolver(case)
    o.set_exact_velocity(0, 0.0, True)
    o.set_exact_pressure(0.0)
    call = make_solver(mg, dict(kw, exact_kind=mg.FIELD_CALLER))
    call.load_state({n: o.get(n) for n in O.FIELD_NAMES})
    scratch = O.OracleSolver(case)
    for k in range(2):
        t = k * kw["dt"]
        feed_stage_data(O, scratch, call, t, kw["dt"], nhn=True)
        call.timestep_nhn(t)
        o.timestep_nhn(t)
    for n in O.FIELD_NAMES:
        assert field_err(n, call.download(n), o.get(n), o.get("p")) <= FP64_TOL, n
    call.close()


def test_standalone_nhn_solve_matches_oracle(oracle_lib, mifgpu_lib, cuda_device):
    """solve_pressure_equation_non_homogeneous_neumann on random velocity and
    Ethier-Steinman gradient data, FP64 and mixed, against the oracle's."""
    O, mg = oracle_lib, mifgpu_lib
    kw = dict(n_global=(9, 27, 45), size=(1.5707963267948966,) * 3, origin=(-1.5707963267948966,) * 3, Re=1.0,
              dt=1.0, exact_kind=2)
    case = O.Case(**kw)
    o = O.OracleSolver(case)
    rng = np.random.default_rng(8)
    st = {n: rng.standard_normal(o.shape(n)) for n in ("u", "v", "w")}
    o.load_state(st)
    o.solve_pressure_nhn(0, 0.5, 0.7, 0.4)
    faces = O.gradient_faces(case, 0.7, 0.4)
    for prec, tol in ((mg.FP64, FP64_TOL), (mg.MIXED, 2e-5)):
        g = make_solver(mg, kw, precision=prec)
        g.load_state(st)
        g.solve_pressure_nhn(0, 0.5, faces)
        assert rel_err(g.download("phi"), o.get("phi")) <= tol, prec
        g.close()


def test_caller_kind_refuses_family_calls(mifgpu_lib, cuda_device):
    mg = mifgpu_lib
    g = make_solver(mg, dict(n_global=(9, 9, 9), exact_kind=mg.FIELD_CALLER))
    for call in (lambda: g.error_norms(0.0), lambda: g.set_exact_velocity(0, 0.0), lambda: g.adjust_pressure(0.0),
                 lambda: g.velocity_error_norms_noalloc(0.0), lambda: g.run(0.0, 2)):
        with pytest.raises(mg.MifGpuError, match=r"\(-4\)"):
            call()
    g.run(0.0, 1)  # one step at a time is fine (zero walls until data is set)
    fam = make_solver(mg, dict(n_global=(9, 9, 9), exact_kind=2))
    u = np.zeros(fam.shape("u"))
    with pytest.raises(mg.MifGpuError, match="MIFGPU_FIELD_CALLER"):
        fam.set_boundary_values(1, u, np.zeros(fam.shape("v")), np.zeros(fam.shape("w")))
    g.close()
    fam.close()
