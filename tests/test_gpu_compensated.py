"""The compensated float state (MIFGPU_MIXED_COMPENSATED), through the C ABI.

Fields and stencils are float as in MIFGPU_MIXED, but every velocity
component of the state carries a bfloat16 residual that keeps what each float
update rounded away, so the state holds about 32 significant bits. These
tests hold it to the FP64 oracle (oracle/mif_oracle.c) much more tightly than
the plain float mode, and check the host boundary (a double uploaded into the
state comes back to ~2^-32 relative) and the paths the mode refuses.
"""
import numpy as np
import pytest

from test_gpu_parity import _oracle_pair, make_solver, rel_err

pytestmark = pytest.mark.gpu


def test_host_roundtrip_keeps_32_bits(mifgpu_lib, cuda_device):
    """Velocity set 0 is split into float + bfloat16 residual on upload and
    summed on download; the pressure and the other sets are plain float."""
    mg = mifgpu_lib
    g = make_solver(mg, dict(n_global=(17, 18, 19)), precision=mg.MIXED_COMPENSATED)
    rng = np.random.default_rng(3)
    for n in ("u", "v", "w"):
        a = rng.standard_normal(g.shape(n)) * 3.0
        g.upload(n, a)
        back = g.download(n)
        assert np.all(np.abs(back - a) <= 2.0 ** -32 * np.abs(a)), n
        # the float part alone would be ~2^-25 off: the residual is really there
        assert np.abs(back - a).max() < 1e-2 * np.abs(a.astype(np.float32) - a).max(), n
    p = rng.standard_normal(g.shape("p"))
    g.upload("p", p)
    assert np.array_equal(g.download("p"), p.astype(np.float32).astype(np.float64))
    g.close()


@pytest.mark.parametrize("shape,periodic,kind", [
    ((33, 33, 33), (False, False, False), 2),
    ((26, 27, 28), (False, True, False), 2),
    ((33, 25, 29), (True, False, True), 0),
    ((32, 33, 30), (True, True, True), 0),
])
def test_compensated_tracks_fp64_oracle(oracle_lib, mifgpu_lib, cuda_device, shape, periodic, kind):
    """Three steps against the FP64 oracle, normwise per field. On the
    smooth manufactured cases (Ethier-Steinman) the compensated state is held
    to 1e-8 of max|u| (the plain float mode is ~1e-7 there and bounded at
    1e-5); on random data, where the first projection removes an O(|u|)
    divergent part through the float Poisson solve, to 2e-6 like the float
    mode."""
    mg = mifgpu_lib
    kw = dict(n_global=shape, size=(1.0, 1.2, 2.0), origin=(0.0, -0.5, -1.0), Re=800.0, dt=2e-4,
              periodic=periodic, exact_kind=kind)
    init = "exact" if kind else "random"
    o, g = _oracle_pair(oracle_lib, mg, kw, precision=mg.MIXED_COMPENSATED, init=init, seed=3)
    _, gm = _oracle_pair(oracle_lib, mg, kw, precision=mg.MIXED, init=init, seed=3)
    for k in range(3):
        o.timestep(k * kw["dt"])
    g.run(0.0, 3)
    gm.run(0.0, 3)
    umax = max(np.abs(o.get(n)).max() for n in "uvw")
    bound = 1e-8 if kind else 2e-6
    for n in ("u", "v", "w"):
        err = rel_err(g.download(n), o.get(n), umax)
        err_mixed = rel_err(gm.download(n), o.get(n), umax)
        assert err <= bound, f"{n}: compensated {err:.3e} (float mode {err_mixed:.3e})"
        if kind:
            assert err < err_mixed, f"{n}: compensated {err:.3e} not below the float mode's {err_mixed:.3e}"
    assert rel_err(g.download("p"), o.get("p")) <= 1e-3
    g.close()
    gm.close()


def test_error_norms_see_the_residual(oracle_lib, mifgpu_lib, cuda_device):
    """error_norms and the allocation-free velocity norms read hi + residual:
    after two steps both equal the oracle's norms (src/Norms.cpp:11-47) of
    the state as downloaded (which is hi + residual in double)."""
    mg = mifgpu_lib
    O = oracle_lib
    kw = dict(n_global=(17, 18, 19), size=(1.0, 1.0, 2.0), origin=(0, 0, -1), Re=1e3, dt=1e-4, exact_kind=2)
    _, g = _oracle_pair(O, mg, kw, precision=mg.MIXED_COMPENSATED)
    g.run(0.0, 2)
    t = 2 * kw["dt"]
    host = O.OracleSolver(O.Case(**kw))
    host.load_state({n: g.download(n) for n in ("u", "v", "w")})
    want = host.error_norms(t)[:3]
    got = g.error_norms(t)[:3]
    np.testing.assert_allclose(got, want, rtol=1e-9)
    np.testing.assert_allclose(g.velocity_error_norms_noalloc(t), got, rtol=1e-12)
    g.close()


def test_compensated_refuses_velocity_only_and_reverse_mode(mifgpu_lib, cuda_device):
    mg = mifgpu_lib
    g = make_solver(mg, dict(n_global=(9, 9, 9), exact_kind=1), precision=mg.MIXED_COMPENSATED)
    with pytest.raises(mg.MifGpuError, match="velocity-only"):
        g.timestep_velocity(0.0)
    with pytest.raises(mg.MifGpuError, match="reverse mode"):
        g.gradient_ke(0.0, 2, 1, (0.0, 1.0, 0.0, 1.0, 0.0, 1.0))
    g.close()


def test_run_hands_projections_between_steps(mifgpu_lib, cuda_device):
    """In a compensated run of several steps each step's last projection is
    applied by the next step's Y2 stage kernel, and the run's last step ends
    with the projection kernel. The state after the run agrees with the same
    steps taken one call at a time (each a complete step) to the float
    rounding of the stencil inputs."""
    mg = mifgpu_lib
    kw = dict(n_global=(33, 34, 35), size=(1.0, 1.0, 2.0), origin=(0.0, 0.0, -1.0), Re=1e3, dt=1e-4, exact_kind=2)
    runs = []
    for chained in (True, False):
        g = make_solver(mg, kw, precision=mg.MIXED_COMPENSATED)
        g.set_exact_velocity(0, 0.0)
        g.set_exact_pressure(0.0)
        if chained:
            g.run(0.0, 5)
        else:
            for k in range(5):
                g.run(k * kw["dt"], 1)
        runs.append({n: g.download(n) for n in ("u", "v", "w", "p")})
        g.close()
    umax = max(np.abs(runs[1][n]).max() for n in "uvw")
    for n in ("u", "v", "w"):
        assert rel_err(runs[0][n], runs[1][n], umax) <= 1e-8, n
    assert rel_err(runs[0]["p"], runs[1]["p"]) <= 1e-5
