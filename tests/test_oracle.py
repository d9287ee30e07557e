"""CPU tests of the oracle: the r2r restatement of FFTW's kinds, the C
restatement of the solver against the reference's own code (bit for bit) and
against the committed golden fixtures, and the manufactured-solution formulas.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN

import sys

sys.path.insert(0, GOLDEN)
from cases import CASES  # noqa: E402


# ---- r2r kinds (FFTW's documented definitions) ----

@pytest.mark.parametrize("n", [2, 3, 4, 5, 7, 8, 9, 16, 17, 20, 38, 65, 97, 129])
def test_redft00_matches_definition_and_scipy(oracle_lib, n):
    rng = np.random.default_rng(n)
    x = rng.standard_normal(n)
    fast = oracle_lib.r2r(3, x)
    direct = oracle_lib.r2r(3, x, direct=True)
    np.testing.assert_allclose(fast, direct, rtol=0, atol=1e-12 * np.abs(direct).max())
    scipy_fft = pytest.importorskip("scipy.fft")
    np.testing.assert_allclose(fast, scipy_fft.dct(x, type=1), rtol=0, atol=1e-12 * np.abs(direct).max())


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 6, 7, 8, 9, 11, 12, 13, 24, 26, 64, 100])
def test_r2hc_hc2r_match_definition_and_roundtrip(oracle_lib, n):
    rng = np.random.default_rng(100 + n)
    x = rng.standard_normal(n)
    hc = oracle_lib.r2r(0, x)
    np.testing.assert_allclose(hc, oracle_lib.r2r(0, x, direct=True), atol=1e-12 * max(1, np.abs(hc).max()))
    # Half-complex order: r_0..r_{n/2}, i_{(n+1)/2-1}..i_1 (numpy rfft for the check)
    X = np.fft.rfft(x)
    want = np.concatenate([X.real[: n // 2 + 1], X.imag[1:(n + 1) // 2][::-1]])
    np.testing.assert_allclose(hc, want, atol=1e-12 * max(1, np.abs(want).max()))
    back = oracle_lib.r2r(1, hc)
    np.testing.assert_allclose(back / n, x, atol=1e-13 * n)
    np.testing.assert_allclose(back, oracle_lib.r2r(1, hc, direct=True), atol=1e-12 * max(1, np.abs(back).max()))


@pytest.mark.parametrize("n", [9, 17, 33, 65])
def test_reference_1d_neumann_known_answer(oracle_lib, n):
    """test/fftw/test_fftw_1d_neumann.cpp: cos(x) on [0, 2 pi] with the DCT-I
    solver, eigenvalues 2 cos(pi k/(N-1)) - 2 and normalisation 2(N-1); the
    error must be O(h^2)."""
    h = 2 * np.pi / (n - 1)
    xex = np.cos(h * np.arange(n))
    bt = oracle_lib.r2r(3, -xex)
    xt = np.zeros(n)
    k = np.arange(1, n)
    xt[1:] = bt[1:] / (2 * np.cos(np.pi * k / (n - 1)) - 2) * h * h
    x = oracle_lib.r2r(3, xt) / (2.0 * (n - 1))
    err = np.abs(xex - x - (xex[0] - x[0])).max()
    assert err < 0.2 * h * h


@pytest.mark.parametrize("n", [8, 16, 32, 64])
def test_reference_1d_periodic_known_answer(oracle_lib, n):
    """test/fftw/test_fftw_1d_periodic.cpp: R2HC/HC2R with normalisation N."""
    h = 2 * np.pi / n
    xex = np.cos(h * np.arange(n))
    bt = oracle_lib.r2r(0, -xex)
    xt = np.zeros(n)
    k = np.arange(1, n)
    xt[1:] = bt[1:] / (2 * np.cos(2 * np.pi * k / n) - 2) * h * h
    x = oracle_lib.r2r(1, xt) / n
    err = np.abs(xex - x - (xex[0] - x[0])).max()
    assert err < 0.2 * h * h


# ---- the C restatement against the golden fixtures (made by the reference itself) ----

def _run_oracle(oracle_lib, spec, fixture):
    O = oracle_lib
    case = O.Case(**spec["case"])
    s = O.OracleSolver(case)
    s.load_state({n: fixture[f"in_{n}"] for n in O.FIELD_NAMES})
    t0 = spec.get("t0", 0.0)
    for k in range(spec.get("steps", 1)):
        t = t0 + k * case.dt
        op = spec["op"]
        if op == "solve_pressure":
            s.solve_pressure(0, spec.get("solve_dt", 1.0))
        elif op == "apply_bc":
            s.apply_bc(0, spec.get("bc_t", 0.3))
        elif op == "solve_pressure_nhn":
            s.solve_pressure_nhn(0, spec.get("solve_dt", 1.0), spec["t_new"], spec["t_old"])
        else:
            getattr(s, op)(t)
    return s, case


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_bit_exact_against_golden(oracle_lib, name):
    fixture = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    spec = CASES[name]
    s, case = _run_oracle(oracle_lib, spec, fixture)
    for n in oracle_lib.FIELD_NAMES:
        got, want = s.get(n), fixture[f"out_{n}"]
        assert np.array_equal(got, want), f"{name}/{n}: max diff {np.abs(got - want).max()}"
    if case.exact_kind:
        t_end = spec.get("t0", 0.0) + spec.get("steps", 1) * case.dt
        np.testing.assert_allclose(s.error_norms(t_end), fixture["norms"], rtol=1e-13, atol=0)


def test_oracle_bit_exact_against_reference_library(oracle_lib):
    """When the reference sources were compiled here, compare directly on a
    larger case than the fixtures hold."""
    O = oracle_lib
    if not O.RefSolver.available():
        pytest.skip("reference library not built here (no reference sources)")
    case = O.Case(n_global=(17, 16, 15), size=(1.0, 1.0, 2.0), origin=(0, 0, -1), Re=1e3, dt=1e-4, exact_kind=2)
    r, o = O.RefSolver(case), O.OracleSolver(case)
    for s in (r, o):
        s.set_exact_velocity(0, 0.0, True)
        s.set_exact_pressure(0.0)
        for k in range(2):
            s.timestep(k * case.dt)
    for n in O.FIELD_NAMES:
        assert np.array_equal(r.get(n), o.get(n)), n


@pytest.mark.parametrize("shape,periodic", [
    ((9, 8, 7), (False, False, False)),
    ((8, 9, 10), (True, True, True)),
    ((9, 7, 8), (True, False, True)),
    ((7, 8, 9), (False, True, False)),
])
def test_oracle_project_bit_exact_against_reference_library(oracle_lib, shape, periodic):
    """p += phi and u -= dt grad(phi) on a velocity set, against the
    reference's update_pressure and update_velocity_pressure_gradient
    (src/Timestep.cpp:66-81). Every field, ghosts included, is random."""
    O = oracle_lib
    if not O.RefSolver.available():
        pytest.skip("reference library not built here (no reference sources)")
    case = O.Case(n_global=shape, size=(1.0, 1.2, 2.0), origin=(0.0, -0.5, -1.0), Re=800.0, dt=2e-4,
                  periodic=periodic)
    r, o = O.RefSolver(case), O.OracleSolver(case)
    rng = np.random.default_rng(17)
    for n in O.FIELD_NAMES:
        a = rng.standard_normal(o.shape(n))
        r.set(n, a)
        o.set(n, a)
    for s in (r, o):
        s.project(1, 3.7e-4)
    for n in O.FIELD_NAMES:
        assert np.array_equal(r.get(n), o.get(n)), n


def test_forcing_formula_matches_symbolic_residual(oracle_lib):
    """The hand-written SINCOS forcing equals u_t + (u.grad)u - lap(u)/Re (+grad p)
    derived symbolically, the construction of generators/manufsol_velocity.py."""
    sp = pytest.importorskip("sympy")
    import ctypes as C

    t, x, y, z = sp.symbols("t x y z")
    Re = 700.0
    u = sp.sin(x) * sp.cos(y) * sp.sin(z) * sp.sin(t)
    v = sp.cos(x) * sp.sin(y) * sp.sin(z) * sp.sin(t)
    w = 2 * sp.cos(x) * sp.cos(y) * sp.cos(z) * sp.sin(t)
    p = sp.cos(x) * sp.cos(y) * sp.sin(z) * sp.sin(t)
    vel = (u, v, w)
    lap = lambda f: sp.diff(f, x, 2) + sp.diff(f, y, 2) + sp.diff(f, z, 2)  # noqa: E731
    res = [sp.diff(c, t) + u * sp.diff(c, x) + v * sp.diff(c, y) + w * sp.diff(c, z) - lap(c) / Re for c in vel]
    grads = [sp.diff(p, a) for a in (x, y, z)]
    assert sp.simplify(sp.diff(u, x) + sp.diff(v, y) + sp.diff(w, z)) == 0
    # evaluate the C formula through a tiny ctypes shim around oracle/manufactured.h
    case = oracle_lib.Case(n_global=(5, 5, 5), exact_kind=1, Re=Re, forcing=2)
    s = oracle_lib.OracleSolver(case)
    rng = np.random.default_rng(0)
    for _ in range(5):
        pt = rng.uniform(-2, 2, 4)
        subs = {t: pt[0], x: pt[1], y: pt[2], z: pt[3]}
        for c in range(3):
            want_v = float(res[c].evalf(subs=subs))
            want_p = float((res[c] + grads[c]).evalf(subs=subs))
            fn = s.lib.mif_oracle_forcing_value
            fn.restype = C.c_double
            fn.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int]
            assert abs(fn(1, c, *pt, Re, 0) - want_v) < 1e-12 * max(1, abs(want_v))
            assert abs(fn(1, c, *pt, Re, 1) - want_p) < 1e-12 * max(1, abs(want_p))


def test_ethier_pressure_gradient_matches_symbolic(oracle_lib):
    sp = pytest.importorskip("sympy")
    import ctypes as C

    t, x, y, z = sp.symbols("t x y z")
    a, d, Re = sp.pi / 4, sp.pi / 2, 1000.0
    p = (-a * a / 2 * (sp.exp(2 * a * x) + sp.exp(2 * a * y) + sp.exp(2 * a * z)
                       + 2 * sp.sin(a * x + d * y) * sp.cos(a * z + d * x) * sp.exp(a * (y + z))
                       + 2 * sp.sin(a * y + d * z) * sp.cos(a * x + d * y) * sp.exp(a * (z + x))
                       + 2 * sp.sin(a * z + d * x) * sp.cos(a * y + d * z) * sp.exp(a * (x + y)))
         * sp.exp(-2 * d * d * t / Re))
    case = oracle_lib.Case(n_global=(5, 5, 5), exact_kind=2, Re=Re)
    s = oracle_lib.OracleSolver(case)
    fn = s.lib.mif_oracle_pressure_gradient_value
    fn.restype = C.c_double
    fn.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double]
    rng = np.random.default_rng(1)
    for _ in range(4):
        pt = rng.uniform(-1, 1, 4)
        subs = {t: pt[0], x: pt[1], y: pt[2], z: pt[3]}
        for c, var in enumerate((x, y, z)):
            want = float(sp.diff(p, var).evalf(subs=subs))
            assert abs(fn(2, c, *pt, Re) - want) < 1e-12 * max(1, abs(want))
