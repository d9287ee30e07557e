"""GPU parity of the CUDA library against the oracle, through the C ABI.

FP64 mode must match within 1e-12 normwise per field (max|gpu - cpu| /
max|cpu|), the required tolerance: the GPU evaluates the same expressions
but may fuse multiply-adds and uses its own FFT, so bits differ by rounding.
Mixed mode is compared with the FP64 oracle at a float tolerance.

phi (pressure_buffer) is the last stage's pressure increment. For a nearly
solenoidal field it is the solution of a Poisson problem whose right-hand
side div(u*)/dt is a small difference of O(|u|/h) terms, so ulp-level input
differences are amplified in its own relative error: perturbing the oracle's
inputs by 2e-16 moves the reference algorithm's phi by ~5e-9 of max|phi| on
the periodic golden case (max|phi| ~ 1e-4 max|p|). phi is therefore compared
on the scale of the pressure it increments, max(|phi|, |p|), still at 1e-12.
"""
import os
import sys

import numpy as np
import pytest

from conftest import GOLDEN

sys.path.insert(0, GOLDEN)
from cases import CASES  # noqa: E402

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12


def rel_err(got, want, scale=None):
    if scale is None:
        scale = np.abs(want).max()
    return np.abs(got - want).max() / max(scale, 1e-300)


def field_err(name, got, want, p_want):
    """Normwise relative error; phi on the pressure's scale (see module doc)."""
    if name == "phi":
        return rel_err(got, want, max(np.abs(want).max(), np.abs(p_want).max()))
    return rel_err(got, want)


def make_solver(mg, case_kw, precision=0, forcing=0):
    c = dict(case_kw)
    return mg.Solver(
        n_global=c["n_global"], size=c.get("size", (1.0, 1.0, 1.0)), origin=c.get("origin", (0.0, 0.0, 0.0)),
        Re=c.get("Re", 1000.0), dt=c.get("dt", 1e-4), periodic=c.get("periodic", (False, False, False)),
        precision=precision, boundary_kind=c.get("exact_kind", 0), forcing=forcing)


def run_op(s, spec, dt):
    t0 = spec.get("t0", 0.0)
    for k in range(spec.get("steps", 1)):
        t = t0 + k * dt
        op = spec["op"]
        if op == "solve_pressure":
            s.solve_pressure(0, spec.get("solve_dt", 1.0))
        elif op == "solve_pressure_nhn":
            import oracle as O

            faces = O.gradient_faces(O.Case(**spec["case"]), spec["t_new"], spec["t_old"])
            s.solve_pressure_nhn(0, spec.get("solve_dt", 1.0), faces)
        elif op == "apply_bc":
            s.apply_bc(0, spec.get("bc_t", 0.3))
        else:
            getattr(s, op)(t)


@pytest.mark.parametrize("name", sorted(CASES))
def test_fp64_matches_golden(mifgpu_lib, cuda_device, name):
    """Every golden case (produced by the reference's own code) in FP64."""
    fixture = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    spec = CASES[name]
    s = make_solver(mifgpu_lib, spec["case"])
    s.load_state({n: fixture[f"in_{n}"] for n in mifgpu_lib.FIELDS})
    run_op(s, spec, spec["case"].get("dt", 1e-4))
    for n in mifgpu_lib.FIELDS:
        want = fixture[f"out_{n}"]
        got = s.download(n)
        assert got.shape == want.shape
        err = field_err(n, got, want, fixture["out_p"])
        assert err <= FP64_TOL, f"{name}/{n}: {err:.3e}"
    if spec["case"].get("exact_kind", 0):
        t_end = spec.get("t0", 0.0) + spec.get("steps", 1) * spec["case"]["dt"]
        np.testing.assert_allclose(s.error_norms(t_end), fixture["norms"], rtol=1e-9, atol=1e-15)


def _oracle_pair(oracle_lib, mg, case_kw, precision=0, forcing=0, init="exact", seed=0, amp=0.1):
    O = oracle_lib
    case = O.Case(**case_kw, forcing=forcing)
    o = O.OracleSolver(case)
    if init == "exact":
        o.set_exact_velocity(0, 0.0, True)
        o.set_exact_pressure(0.0)
    else:
        rng = np.random.default_rng(seed)
        for n in ("u", "v", "w", "p"):
            o.set(n, rng.standard_normal(o.shape(n)) * amp)
    g = make_solver(mg, case_kw, precision, forcing)
    g.load_state({n: o.get(n) for n in O.FIELD_NAMES})
    return o, g


@pytest.mark.parametrize("shape,periodic,kind", [
    ((33, 34, 35), (False, False, False), 2),
    ((32, 33, 30), (True, True, True), 0),
    ((33, 25, 29), (True, False, True), 0),
    ((26, 27, 28), (False, True, False), 2),
    # the smallest grids the library accepts: 3 points (DCT-I of 3 points,
    # a one-point interior), 3-point periodic axes (real DFT of length 2)
    ((3, 3, 3), (False, False, False), 2),
    ((3, 3, 3), (False, False, False), 0),
    ((4, 3, 5), (True, False, True), 0),
    ((3, 4, 3), (True, True, True), 0),
    ((5, 3, 4), (False, True, False), 2),
])
def test_fp64_steps_match_oracle(oracle_lib, mifgpu_lib, cuda_device, shape, periodic, kind):
    """Three steps in FP64. The bound per field is 1e-12, or four times the
    reference algorithm's own response to a one-ulp perturbation of its
    inputs where that is larger: on the 3 x 4 x 3 periodic grid with random,
    far from solenoidal data phi is 1e-5 of p, and the oracle alone moves
    phi by ~9e-13 (of p's scale) under such a perturbation."""
    kw = dict(n_global=shape, size=(1.0, 1.2, 2.0), origin=(0.0, -0.5, -1.0), Re=800.0, dt=2e-4,
              periodic=periodic, exact_kind=kind)
    init = "exact" if kind else "random"
    o, g = _oracle_pair(oracle_lib, mifgpu_lib, kw, init=init, seed=3)
    inputs = {n: o.get(n).copy() for n in oracle_lib.FIELD_NAMES}
    for k in range(3):
        o.timestep(k * kw["dt"])
    want = {n: o.get(n) for n in oracle_lib.FIELD_NAMES}
    sens = {n: 0.0 for n in want}
    for ps in (1, 2):  # the oracle's one-ulp sensitivity
        rng = np.random.default_rng(100 + ps)
        o2 = oracle_lib.OracleSolver(oracle_lib.Case(**kw))
        for n, a in inputs.items():
            o2.set(n, a * (1.0 + 2.2e-16 * rng.standard_normal(a.shape)))
        for k in range(3):
            o2.timestep(k * kw["dt"])
        for n in want:
            sens[n] = max(sens[n], field_err(n, o2.get(n), want[n], want["p"]))
    g.run(0.0, 3)  # graph replays
    for n in oracle_lib.FIELD_NAMES:
        err = field_err(n, g.download(n), want[n], want["p"])
        assert err <= max(FP64_TOL, 4.0 * sens[n]), f"{n}: {err:.3e} (oracle one-ulp sensitivity {sens[n]:.3e})"


@pytest.mark.parametrize("shape,periodic", [
    ((9, 8, 7), (False, False, False)),
    ((8, 9, 10), (True, True, True)),
    ((9, 7, 8), (True, False, True)),
    ((7, 8, 9), (False, True, False)),
])
def test_project_matches_oracle(oracle_lib, mifgpu_lib, cuda_device, shape, periodic):
    """mifgpu_project on its own (p += phi, then u -= dt grad(phi) on the
    interior of one velocity set, src/Timestep.cpp:66-81). Every field is
    random, ghosts included, so the points it must leave alone are checked
    too."""
    kw = dict(n_global=shape, size=(1.0, 1.2, 2.0), origin=(0.0, -0.5, -1.0), Re=800.0, dt=2e-4,
              periodic=periodic, exact_kind=0)
    o = oracle_lib.OracleSolver(oracle_lib.Case(**kw))
    rng = np.random.default_rng(17)
    for n in oracle_lib.FIELD_NAMES:
        o.set(n, rng.standard_normal(o.shape(n)))
    g = make_solver(mifgpu_lib, kw)
    g.load_state({n: o.get(n) for n in oracle_lib.FIELD_NAMES})
    o.project(1, 3.7e-4)
    g.project(1, 3.7e-4)
    for n in oracle_lib.FIELD_NAMES:
        err = rel_err(g.download(n), o.get(n))
        assert err <= FP64_TOL, f"{n}: {err:.3e}"
    g.close()


def test_contexts_of_different_sizes_coexist(oracle_lib, mifgpu_lib, cuda_device):
    """A context whose line kernels need more dynamic shared memory keeps
    working after a smaller context was created (the kernel attribute is
    process-wide and only ever raised)."""
    kw = dict(n_global=(17, 18, 257), size=(1.0, 1.0, 2.0), Re=500.0, dt=1e-4, exact_kind=2)
    o, big = _oracle_pair(oracle_lib, mifgpu_lib, kw)
    small = make_solver(mifgpu_lib, dict(n_global=(9, 9, 9), exact_kind=2))
    small.set_exact_velocity(0, 0.0)
    small.run(0.0, 1)
    big.run(0.0, 2)
    for k in range(2):
        o.timestep(k * kw["dt"])
    for n in oracle_lib.FIELD_NAMES:
        assert field_err(n, big.download(n), o.get(n), o.get("p")) <= FP64_TOL, n


def test_forcing_extension_matches_oracle(oracle_lib, mifgpu_lib, cuda_device):
    """Projection step with the SINCOS Navier-Stokes forcing (the labelled
    extension for manufactured-solution runs)."""
    kw = dict(n_global=(25, 26, 27), size=(1.0, 1.0, 1.0), Re=1000.0, dt=1e-4, exact_kind=1)
    o, g = _oracle_pair(oracle_lib, mifgpu_lib, kw, forcing=2)
    for k in range(2):
        o.timestep(0.3 + k * kw["dt"])
        g.timestep(0.3 + k * kw["dt"])
    for n in oracle_lib.FIELD_NAMES:
        assert field_err(n, g.download(n), o.get(n), o.get("p")) <= FP64_TOL, n


def test_timestep_host_matches_oracle(oracle_lib, mifgpu_lib, cuda_device):
    """The drop-in form: host buffers in, host buffers out."""
    kw = dict(n_global=(20, 19, 18), size=(1.0, 1.0, 2.0), origin=(0, 0, -1), Re=1e3, dt=1e-4, exact_kind=2)
    o, g = _oracle_pair(oracle_lib, mifgpu_lib, kw)
    u, v, w, p = (np.ascontiguousarray(o.get(n)) for n in ("u", "v", "w", "p"))
    for k in range(2):
        g.timestep_host(k * kw["dt"], u, v, w, p)
        o.timestep(k * kw["dt"])
    for n, a in zip(("u", "v", "w", "p"), (u, v, w, p)):
        assert rel_err(a, o.get(n)) <= FP64_TOL, n


def test_upload_download_roundtrip_over_many_chunks(mifgpu_lib, cuda_device):
    """Fields of ~9.3 M doubles (74 MB) travel as two 64 MB-chunk copies on
    different copy streams; an FP64 context must give every value back bit
    for bit. (Several fields queued at once: test_timestep_host_matches_oracle.)"""
    g = make_solver(mifgpu_lib, dict(n_global=(210, 209, 211)))
    rng = np.random.default_rng(7)
    names = ("u", "v", "w", "p")
    want = {n: rng.standard_normal(g.shape(n)) for n in names}
    assert all(a.size * 8 > 64 << 20 for a in want.values())
    for n in names:
        g.upload(n, want[n])
    for n in names:
        assert np.array_equal(g.download(n), want[n]), n
    g.close()


def test_norms_and_adjust_pressure_match_oracle(oracle_lib, mifgpu_lib, cuda_device):
    kw = dict(n_global=(17, 18, 19), size=(1.0, 1.0, 2.0), origin=(0, 0, -1), Re=1e3, dt=1e-4, exact_kind=2)
    o, g = _oracle_pair(oracle_lib, mifgpu_lib, kw)
    for k in range(2):
        o.timestep(k * kw["dt"])
    g.run(0.0, 2)
    t = 2 * kw["dt"]
    o.adjust_pressure(t)
    g.adjust_pressure(t)
    assert rel_err(g.download("p"), o.get("p")) <= FP64_TOL
    np.testing.assert_allclose(g.error_norms(t), o.error_norms(t), rtol=1e-9)


def test_mixed_precision_tracks_fp64(oracle_lib, mifgpu_lib, cuda_device):
    """FP32 storage and stencils, FP64 eigenvalue division: within float
    rounding of the FP64 result on a smooth manufactured case."""
    kw = dict(n_global=(33, 33, 33), size=(1.0, 1.0, 2.0), origin=(0, 0, -1), Re=1e3, dt=1e-4, exact_kind=2)
    o, g = _oracle_pair(oracle_lib, mifgpu_lib, kw, precision=1)
    for k in range(2):
        o.timestep(k * kw["dt"])
    g.run(0.0, 2)
    for n in ("u", "v", "w"):
        assert rel_err(g.download(n), o.get(n)) <= 1e-5, n
    # the pressure is accumulated from divergences divided by dt: looser
    assert rel_err(g.download("p"), o.get("p")) <= 1e-3


@pytest.mark.parametrize("shape,periodic,kind", [
    ((3, 3, 3), (False, False, False), 2),
    ((5, 3, 4), (False, True, False), 2),
    ((4, 3, 5), (True, False, True), 0),
    ((3, 4, 3), (True, True, True), 0),
])
def test_mixed_precision_on_the_smallest_grids(oracle_lib, mifgpu_lib, cuda_device, shape, periodic, kind):
    """Mixed precision at the smallest accepted sizes (3-point DCT-I lines,
    length-2 real DFTs, all on the shared-memory engine): within float
    rounding of the FP64 oracle, normwise."""
    kw = dict(n_global=shape, size=(1.0, 1.2, 2.0), origin=(0.0, -0.5, -1.0), Re=800.0, dt=2e-4,
              periodic=periodic, exact_kind=kind)
    o, g = _oracle_pair(oracle_lib, mifgpu_lib, kw, precision=1, init="exact" if kind else "random", seed=3)
    for k in range(2):
        o.timestep(k * kw["dt"])
    g.run(0.0, 2)
    for n in ("u", "v", "w"):
        assert rel_err(g.download(n), o.get(n)) <= 1e-5, n
    assert rel_err(g.download("p"), o.get("p")) <= 1e-3


def test_poisson_solution_satisfies_discrete_laplacian(mifgpu_lib, cuda_device):
    """Size-independent property at a larger size: the solve inverts the
    7-point Laplacian with mirror (Neumann) or wrap (periodic) closure, up to
    the removed zero mode."""
    for periodic in ((False, False, False), (True, False, True)):
        n = (65, 49, 57) if not periodic[0] else (65, 49, 65)
        g = mifgpu_lib.Solver(n_global=n, size=(1.0, 0.8, 1.1), periodic=periodic, dt=1.0)
        rng = np.random.default_rng(4)
        for c in ("u", "v", "w"):
            g.upload(c, rng.standard_normal(g.shape(c)))
        g.divergence(0, 1.0)
        ex = g.extent("phi")
        lo = [1 if p else 0 for p in periodic]
        hi = [ex[d] - 1 if periodic[d] else ex[d] for d in range(3)]
        rhs = g.download("phi")[lo[2]:hi[2], lo[1]:hi[1], lo[0]:hi[0]]
        g.solve_pressure(0, 1.0)
        phi = g.download("phi")[lo[2]:hi[2], lo[1]:hi[1], lo[0]:hi[0]]
        h = [1.0 / (n[0] - 1), 0.8 / (n[1] - 1), 1.1 / (n[2] - 1)]
        lap = np.zeros_like(phi)
        for ax, d in ((2, 0), (1, 1), (0, 2)):  # numpy axis, physical axis
            if periodic[d]:
                up, dn = np.roll(phi, -1, ax), np.roll(phi, 1, ax)
            else:
                pad = np.concatenate([np.take(phi, [1], ax), phi, np.take(phi, [-2], ax)], ax)
                up = np.take(pad, range(2, pad.shape[ax]), ax)
                dn = np.take(pad, range(0, pad.shape[ax] - 2), ax)
            lap += (up - 2 * phi + dn) / h[d] ** 2
        resid = lap - rhs
        # the residual is the removed constant mode: constant everywhere
        assert np.abs(resid - resid.mean()).max() <= 1e-9 * np.abs(rhs).max()


@pytest.mark.parametrize("shape,periodic", [
    # a DCT-I line of n points runs on the register path as a length n-1 transform
    ((33, 65, 129), (False, False, False)),   # DCT-I: shared-memory 64 / register 64, 128 (z fused)
    ((257, 17, 33), (False, False, False)),   # register 256
    ((513, 9, 17), (False, False, False)),    # register 512
    ((1025, 9, 5), (False, False, False)),    # register 1024
    ((65, 129, 33), (True, True, True)),      # real DFT lengths 64, 128, 32 (32: shared-memory path)
    ((257, 65, 513), (True, False, True)),    # channel-like: real DFT 256 / DCT 64 / real DFT 512
    ((17, 513, 9), (False, False, False)),    # register 512 along the strided y axis
    ((769, 9, 5), (False, False, False)),     # register 768 = 48 x 16 (radix-3 base) along x
    ((5, 9, 385), (False, False, False)),     # register 384 = 48 x 8, z fused
    ((9, 769, 5), (False, True, False)),      # real DFT 768 along the strided y axis
    ((9, 5, 385), (False, False, True)),      # real DFT 384, z fused
    # strided DCT-I lines staged by TMA in groups of four lines from an odd x
    # origin (periodic x: lead 1), 513 points in three boxes
    ((32, 513, 9), (True, False, False)),     # y sweeps
    ((9, 17, 513), (True, False, False)),     # the fused z sweep
])
def test_mixed_poisson_matches_oracle(oracle_lib, mifgpu_lib, cuda_device, shape, periodic):
    """Mixed-precision Poisson solve (register FFT for power-of-two lengths)
    against the FP64 oracle on a random right-hand side."""
    O = oracle_lib
    case = O.Case(n_global=shape, size=(1.0, 0.7, 1.3), periodic=periodic, dt=1.0)
    o = O.OracleSolver(case)
    rng = np.random.default_rng(sum(shape))
    st = {c: rng.standard_normal(o.shape(c)) for c in ("u", "v", "w")}
    o.load_state(st)
    o.solve_pressure(0, 0.5)
    g = make_solver(mifgpu_lib, dict(n_global=shape, size=(1.0, 0.7, 1.3), periodic=periodic, dt=1.0), precision=1)
    g.load_state(st)
    g.solve_pressure(0, 0.5)
    want = o.get("phi")
    assert rel_err(g.download("phi"), want) <= 2e-5


def test_nonfinite_watchdog(mifgpu_lib, cuda_device):
    """A NaN placed in the velocity from the host reaches every value of the
    pressure increment; the step reports MIFGPU_ENONFINITE (-5), also through
    the drop-in host call, and a clean state steps normally again."""
    mg = mifgpu_lib
    for prec in (mg.FP64, mg.MIXED, mg.MIXED_COMPENSATED):
        g = make_solver(mg, dict(n_global=(17, 18, 19), exact_kind=2), precision=prec)
        g.set_exact_velocity(0, 0.0)
        g.set_exact_pressure(0.0)
        g.run(0.0, 1)
        clean = {n: g.download(n) for n in ("u", "v", "w", "p")}
        bad = clean["v"].copy()
        bad[5, 6, 7] = np.nan
        g.upload("v", bad)
        with pytest.raises(mg.MifGpuError, match=r"\(-5\).*NaN or Inf"):
            g.run(1e-4, 2)
        arrs = [clean[n].copy() for n in ("u", "v", "w", "p")]  # timestep_host writes into them
        arrs[2][3, 3, 3] = np.inf
        with pytest.raises(mg.MifGpuError, match=r"\(-5\)"):
            g.timestep_host(1e-4, *arrs)
        assert not np.isfinite(arrs[0]).all()  # the non-finite state came back to the host
        g.load_state(clean)
        g.run(1e-4, 2)
        assert all(np.isfinite(g.download(n)).all() for n in ("u", "v", "w", "p"))
        g.close()


def test_run_velocity_matches_single_steps_and_oracle(oracle_lib, mifgpu_lib, cuda_device):
    """mifgpu_run_velocity (graph replays with the set swap inside the run)
    gives the fields of the same number of mifgpu_timestep_velocity calls bit
    for bit, and follows the oracle's timestep_velocity
    (src/TimestepVelocity.cpp:60-90) within 1e-12 over an odd and an even
    number of steps (the swap leaves the state in either labelling)."""
    mg = mifgpu_lib
    kw = dict(n_global=(21, 22, 23), size=(1.0, 1.0, 1.0), Re=1e4, dt=1e-4, exact_kind=1)
    for nsteps in (4, 5):
        o, g1 = _oracle_pair(oracle_lib, mg, kw, forcing=1)
        _, g2 = _oracle_pair(oracle_lib, mg, kw, forcing=1)
        for k in range(nsteps):
            t = 0.25 + k * kw["dt"]
            o.timestep_velocity(t)
            g1.timestep_velocity(t)
        g2.run_velocity(0.25, nsteps)
        for n in ("u", "v", "w", "u1", "v1", "w1"):
            assert np.array_equal(g1.download(n), g2.download(n)), (nsteps, n)
            assert rel_err(g2.download(n), o.get(n)) <= FP64_TOL, (nsteps, n)
        g1.close()
        g2.close()
