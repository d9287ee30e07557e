"""GPU parity at the benchmark configurations' own sizes, through the C ABI.

Three of the reference's benchmark workloads run step by step on the CUDA
library and on the oracle (oracle/mif_oracle.c, the bit-exact restatement of
src/Timestep.cpp:97-141) from identical inputs:

* the 64^3-cell manufactured cube (65^3 nodes), SINCOS velocity with the
  Navier-Stokes forcing extension, Re 1000, dt 1e-4, all 10 steps;
* the periodic 128^3 box (129^3 nodes, [0, 2pi]^3) from the seeded k^-2
  solenoidal field of the adjoint workload (|k| <= 8, max |u| = 1), Re 500,
  dt 2e-3, three steps, no forcing;
* the boundary-layer channel geometry ([0, 4pi] x [0, 2] x [0, 2pi], periodic
  x and z, no-slip walls in y) at a quarter of its size per axis, 128 x 64 x
  128 cells with the same aspect, laminar profile plus seeded 1e-2 solenoidal
  noise, Re 5000, dt 5e-4, three steps.

FP64 is held to 1e-12 per field per step (normwise, max|gpu - cpu| / max|cpu|),
or to four times the oracle's own response to a one-ulp perturbation of its
inputs and of its forcing values where that is larger (phi, the last stage's
pressure increment, is measured on the scale of the pressure it increments;
see test_gpu_parity.py). The velocity is held to 1e-12 outright. On the
manufactured cube, which starts from rest, p after the first step is the sum
of three phi and inherits their conditioning: the oracle alone moves it by
8.8e-13 of max|p| under one-ulp forcing noise.
Mixed precision is held to the FP64 oracle at the float bounds stated in each
test. The inputs come from the benchmark's own generators (bench.py).
"""
import math

import numpy as np
import pytest

from bench import random_solenoidal, solenoidal_noise, staggered_coords

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
PI = math.pi


def rel_err(got, want, scale=None):
    if scale is None:
        scale = np.abs(want).max()
    return float(np.abs(got - want).max() / max(scale, 1e-300))


def field_err(name, got, want, p_want):
    if name == "phi":
        return rel_err(got, want, max(np.abs(want).max(), np.abs(p_want).max()))
    return rel_err(got, want)


CONFIGS = {
    "config1_cube64_sincos": dict(
        case=dict(n_global=(65, 65, 65), size=(1.0, 1.0, 1.0), Re=1000.0, dt=1e-4, exact_kind=1),
        forcing=2, steps=10, init="exact"),
    "config4_periodic128": dict(
        case=dict(n_global=(129, 129, 129), size=(2 * PI,) * 3, Re=500.0, dt=2e-3, periodic=(True, True, True)),
        forcing=0, steps=3, init="k2_field"),
    "config3_channel128x64x128": dict(
        case=dict(n_global=(129, 65, 129), size=(4 * PI, 2.0, 2 * PI), Re=5000.0, dt=5e-4,
                  periodic=(True, False, True)),
        forcing=0, steps=3, init="channel"),
}


def initial_state(O, o, spec):
    """Inputs of one configuration in the reference layout (numpy arrays)."""
    c = spec["case"]
    if spec["init"] == "exact":
        o.set_exact_velocity(0, 0.0, True)
        o.set_exact_pressure(0.0)
        return {n: o.get(n) for n in ("u", "v", "w", "p")}
    if spec["init"] == "k2_field":
        n = c["n_global"][0] - 1
        st = random_solenoidal(o.shape, n, c["size"][0], 8, 1.0, 1234)
    else:
        ncell = tuple(c["n_global"][d] - 1 for d in range(3))
        noise = solenoidal_noise(o.shape, ncell, c["size"], (-1, 0, -1), 16, 1e-2, 12)
        st = {}
        for nm in "uvw":
            x, y, z = staggered_coords(o, nm, c["n_global"], c["size"], (0.0,) * 3, c["periodic"])
            st[nm] = (1.0 - (y - 1.0) ** 2 if nm == "u" else 0.0 * y) + noise[nm]
    st["p"] = np.zeros(o.shape("p"))
    return st


def make_pair(O, mg, spec, precision):
    c = spec["case"]
    case = O.Case(**c, forcing=spec["forcing"])
    o = O.OracleSolver(case)
    st = initial_state(O, o, spec)
    o.load_state(st)
    g = mg.Solver(n_global=c["n_global"], size=c["size"], Re=c["Re"], dt=c["dt"],
                  periodic=c.get("periodic", (False, False, False)), precision=precision,
                  boundary_kind=c.get("exact_kind", 0), forcing=spec["forcing"])
    g.load_state(st)
    return case, o, g, st


def oracle_sensitivity(O, case, st, steps):
    """An oracle run whose inputs, and every forcing value it evaluates, carry
    a one-ulp relative perturbation: its distance from the unperturbed run is
    the reference algorithm's own response to rounding. (The manufactured
    cube starts from a zero state, where only the forcing has values to
    perturb; the GPU evaluates that forcing from sin/cos tables with fused
    multiply-adds, one-ulp different per point.)"""
    rng = np.random.default_rng(101)
    o = O.OracleSolver(case)
    o.load_state({n: a * (1.0 + 2.2e-16 * rng.standard_normal(a.shape)) for n, a in st.items()})
    if case.forcing:
        o.set_forcing_noise(2.2e-16, 7)
    return o


@pytest.mark.parametrize("name", sorted(CONFIGS))
def test_config_fp64_matches_oracle_every_step(oracle_lib, mifgpu_lib, cuda_device, name):
    spec = CONFIGS[name]
    O = oracle_lib
    case, o, g, st = make_pair(O, mifgpu_lib, spec, mifgpu_lib.FP64)
    o_pert = oracle_sensitivity(O, case, st, spec["steps"])
    dt = spec["case"]["dt"]
    worst = {}
    for k in range(spec["steps"]):
        t = k * dt
        o.timestep(t)
        o_pert.timestep(t)
        g.timestep(t)
        want = {n: o.get(n) for n in O.FIELD_NAMES}
        for n in O.FIELD_NAMES:
            sens = field_err(n, o_pert.get(n), want[n], want["p"])
            err = field_err(n, g.download(n), want[n], want["p"])
            bound = max(FP64_TOL, 4.0 * sens)
            assert err <= bound, f"{name} step {k + 1} {n}: {err:.3e} > {bound:.3e} (oracle one-ulp {sens:.3e})"
            worst[n] = max(worst.get(n, 0.0), err)
    g.close()
    # the velocity, the state the step advances, is within 1e-12 outright
    for n in ("u", "v", "w"):
        assert worst[n] <= FP64_TOL, (n, worst[n])


# The float modes against the FP64 oracle after the whole window, normwise.
# MIXED: velocity within 2e-6 of max|u| (float storage rounding accumulated
# over the steps). MIXED_COMPENSATED: within 2e-7 (the state keeps ~32 bits;
# what is left is the float right-hand sides and Poisson solves). The
# pressure within 1e-3 of max|p| in both: it is a sum of float divergences
# divided by dt, and on the manufactured cube, which starts from rest, max|p|
# is only 5e-4 after the ten steps.
FLOAT_BOUNDS = {"mixed": {"velocity": 2e-6, "p": 1e-3}, "compensated": {"velocity": 2e-7, "p": 1e-3}}
_ORACLE_FINAL = {}


@pytest.mark.parametrize("mode", ["mixed", "compensated"])
@pytest.mark.parametrize("name", sorted(CONFIGS))
def test_config_float_modes_track_fp64_oracle(oracle_lib, mifgpu_lib, cuda_device, name, mode):
    spec = CONFIGS[name]
    O = oracle_lib
    mg = mifgpu_lib
    prec = mg.MIXED if mode == "mixed" else mg.MIXED_COMPENSATED
    case, o, g, st = make_pair(O, mg, spec, prec)
    dt = spec["case"]["dt"]
    if name not in _ORACLE_FINAL:  # the FP64 oracle's state after the window, once per configuration
        for k in range(spec["steps"]):
            o.timestep(k * dt)
        _ORACLE_FINAL[name] = {n: o.get(n) for n in ("u", "v", "w", "p")}
    want = _ORACLE_FINAL[name]
    g.run(0.0, spec["steps"])
    umax = max(np.abs(want[n]).max() for n in "uvw")
    errs = {n: rel_err(g.download(n), want[n], umax) for n in "uvw"}
    errs["p"] = rel_err(g.download("p"), want["p"])
    print(f"{name} {mode}: " + " ".join(f"{n} {e:.3e}" for n, e in errs.items()))
    for n in "uvw":
        assert errs[n] <= FLOAT_BOUNDS[mode]["velocity"], f"{name} {mode} {n}: {errs[n]:.3e}"
    assert errs["p"] <= FLOAT_BOUNDS[mode]["p"], f"{name} {mode} p: {errs['p']:.3e}"
    g.close()
