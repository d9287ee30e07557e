"""mifgpu_velocity_error_norms_noalloc: the velocity error norms from the
library's static device scratch, compared with mifgpu_error_norms (the entry
point that reduces into context memory) on two calls in a row. Collected last
so that it also runs after every other GPU test of the session."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def make(mg, n_global, precision, periodic=(False, False, False), kind=1):
    return mg.Solver(n_global=n_global, Re=1000.0, dt=1e-4, periodic=periodic, precision=precision,
                     boundary_kind=kind, forcing=mg.FORCING_NAVIER_STOKES)


@pytest.mark.parametrize("precision", [0, 1, 2], ids=["fp64", "mixed", "compensated"])
@pytest.mark.parametrize("periodic,kind", [((False, False, False), 1), ((True, False, True), 2)],
                         ids=["dirichlet", "periodic_xz"])
def test_noalloc_norms_match_error_norms(mifgpu_lib, cuda_device, precision, periodic, kind):
    """Dirichlet box with the SINCOS family, and a box periodic in x and z
    (interior index ranges shifted by the ghosts) with the Ethier-Steinman
    family; every precision, the compensated one reading hi + residual."""
    mg = mifgpu_lib
    s = make(mg, (17, 18, 19), precision, periodic=periodic, kind=kind)
    s.set_exact_velocity(0, 0.3)
    s.set_exact_pressure(0.3)
    rng = np.random.default_rng(2)
    u = s.download("u")
    s.upload("u", u + 1e-3 * rng.standard_normal(u.shape))
    s.run(0.3, 2)
    t = 0.3 + 2 * 1e-4
    want = s.error_norms(t)[:3]
    first = s.velocity_error_norms_noalloc(t)
    second = s.velocity_error_norms_noalloc(t)
    np.testing.assert_array_equal(first, second)  # fixed reduction order
    # the two entry points' per-point arithmetic is compiled separately (its
    # multiply-adds may contract differently), so even the maximum agrees to
    # rounding, not bit for bit
    np.testing.assert_allclose(first, want, rtol=1e-12, atol=0)
    s.close()


@pytest.mark.parametrize("precision", [0, 2], ids=["fp64", "compensated"])
def test_noalloc_norms_split_flat_planes(mifgpu_lib, cuda_device, precision):
    """A flat grid (three interior planes of 127 x 128 points): each plane is
    split into 15 chunks, the last one short, and the result still matches
    error_norms and repeats bit for bit."""
    mg = mifgpu_lib
    s = make(mg, (129, 130, 5), precision, kind=1)
    s.set_exact_velocity(0, 0.3)
    rng = np.random.default_rng(5)
    for name in ("u", "v", "w"):
        f = s.download(name)
        s.upload(name, f + 1e-3 * rng.standard_normal(f.shape))
    want = s.error_norms(0.3)[:3]
    first = s.velocity_error_norms_noalloc(0.3)
    second = s.velocity_error_norms_noalloc(0.3)
    np.testing.assert_array_equal(first, second)
    np.testing.assert_allclose(first, want, rtol=1e-12, atol=0)
    s.close()


def test_noalloc_norms_reject_too_many_planes(mifgpu_lib, cuda_device):
    """A z extent of 4098 points (4096 interior planes) exceeds the 4000-plane scratch."""
    mg = mifgpu_lib
    s = make(mg, (5, 5, 4097), 0, periodic=(False, False, True), kind=0)
    with pytest.raises(mg.MifGpuError, match="4000"):
        s.velocity_error_norms_noalloc(0.0)
    s.close()
