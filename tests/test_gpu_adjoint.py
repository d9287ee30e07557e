"""Reverse mode of the projection step (mifgpu_gradient_ke / mifgpu_backward).

The reference has no adjoint, so there is no oracle to compare with: the
gradient is checked against the library's own forward map, in FP64, by
  * central finite differences at single grid values of the initial u, v,
    w, p (interior, ghost and wall points); one grid value moves the loss
    so little that the step is 1e-4 there, to stay clear of the loss's
    rounding noise (the map is smooth: the O(eps^2) truncation stays far
    below the tolerance),
  * the dot-product test: <adjoint, delta> against the tangent-linear
    derivative of the loss along a random delta (central difference,
    eps = 1e-6),
  * the derivative with respect to the Taylor-Green forcing amplitude
    (step 1e-4),
each to a relative error of 1e-6 (the required bound), on a periodic box,
an all-Dirichlet box with time-dependent wall data and a channel. The FP32
adjoint is compared with the FP64 one; the checkpoint interval must not
change the result; the autograd wrapper must return the same gradient.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

EPS = 1e-6
EPS_POINT = 1e-4
TOL = 1e-6

CASES = {
    # periodic box, Taylor-Green forcing, loss box in the middle
    "periodic": dict(n_global=(17, 17, 17), size=(2 * math.pi,) * 3, periodic=(True, True, True), Re=100.0,
                     dt=1e-2, kind=0, alpha=0.3, nsteps=5, every=2, t0=0.0,
                     box=(math.pi / 2, 3 * math.pi / 2) * 3),
    # all walls with the SINCOS wall data (time dependent), DCT pressure
    "dirichlet": dict(n_global=(10, 11, 12), size=(1.0, 1.0, 1.0), periodic=(False, False, False), Re=50.0,
                      dt=2e-3, kind=1, alpha=0.2, nsteps=4, every=3, t0=0.5,
                      box=(0.25, 0.8, 0.1, 0.9, 0.3, 0.7)),
    # channel: periodic x and z, walls in y
    "channel": dict(n_global=(13, 9, 11), size=(2 * math.pi, 2.0, math.pi), origin=(0.0, -1.0, 0.0),
                    periodic=(True, False, True), Re=80.0, dt=5e-3, kind=0, alpha=0.25, nsteps=3, every=1,
                    t0=0.0, box=(1.0, 5.0, -0.5, 0.5, 0.5, 2.5)),
}


def coords(c, comp, shape):
    """Positions of component comp's staggered points (reference layout (z, y, x))."""
    out = []
    for d in range(3):
        n = c["n_global"][d]
        per = c["periodic"][d]
        h = c["size"][d] / (n - 1)
        base = -1 if per else 0
        ext = shape[2 - d]
        x = c.get("origin", (0.0, 0.0, 0.0))[d] + h * (base + np.arange(ext))
        if d == comp:
            x = x - h / 2
        out.append(x)
    z, y, x = np.meshgrid(out[2], out[1], out[0], indexing="ij")
    return x, y, z


def smooth_field(c, comp, shape, rng):
    """A few random periodic modes (|k| <= 2) plus the Taylor-Green pattern."""
    x, y, z = coords(c, comp, shape)
    L = c["size"]
    f = np.zeros(shape)
    if comp == 0:
        f += np.sin(2 * math.pi * x / L[0]) * np.cos(2 * math.pi * y / L[1]) * np.cos(2 * math.pi * z / L[2])
    elif comp == 1:
        f -= np.cos(2 * math.pi * x / L[0]) * np.sin(2 * math.pi * y / L[1]) * np.cos(2 * math.pi * z / L[2])
    for _ in range(4):
        k = rng.integers(-2, 3, size=3)
        ph = rng.uniform(0, 2 * math.pi)
        f += 0.1 * rng.standard_normal() * np.sin(
            2 * math.pi * (k[0] * x / L[0] + k[1] * y / L[1] + k[2] * z / L[2]) + ph)
    return f


def make(mg, c, precision):
    return mg.Solver(n_global=c["n_global"], size=c["size"], origin=c.get("origin", (0.0, 0.0, 0.0)), Re=c["Re"],
                     dt=c["dt"], periodic=c["periodic"], precision=precision, boundary_kind=c["kind"],
                     forcing=mg.FORCING_TAYLOR_GREEN, forcing_amplitude=c["alpha"])


def initial_state(s, c):
    rng = np.random.default_rng(7)
    st = {}
    for comp, n in enumerate("uvw"):
        st[n] = smooth_field(c, comp, s.shape(n), rng)
    st["p"] = 0.1 * smooth_field(c, 2, s.shape("p"), rng)
    return st


def loss_and_grad(s, c, st, alpha=None, every=None):
    s.set_forcing_amplitude(c["alpha"] if alpha is None else alpha)
    s.load_state(st)
    r = s.gradient_ke(c["t0"], c["nsteps"], every or c["every"], c["box"])
    return r, {n: s.adjoint(n) for n in "uvwp"}


def loss_only(s, c, st, alpha=None):
    return loss_and_grad(s, c, st, alpha)[0]["loss"]


def ke_numpy(s, c):
    vol = np.prod([c["size"][d] / (c["n_global"][d] - 1) for d in range(3)])
    x0, x1, y0, y1, z0, z1 = c["box"]
    tot = 0.0
    for comp, n in enumerate("uvw"):
        a = s.download(n)
        x, y, z = coords(c, comp, a.shape)
        m = np.zeros(a.shape, bool)
        m[1:-1, 1:-1, 1:-1] = True
        m &= (x >= x0) & (x <= x1) & (y >= y0) & (y <= y1) & (z >= z0) & (z <= z1)
        tot += 0.5 * vol * np.sum(a[m] ** 2)
    return tot


def probe_points(shape, rng):
    """Interior points and points on each boundary layer (ghost or wall)."""
    ez, ey, ex = shape
    pts = [(ez // 2, ey // 2, ex // 2), (1, 1, 1), (ez - 2, ey - 2, ex - 2)]
    pts += [(0, ey // 2, ex // 3), (ez // 3, ey - 1, ex // 2), (ez // 2, ey // 3, 0), (ez // 2, ey // 2, ex - 1)]
    pts += [tuple(int(rng.integers(0, e)) for e in shape) for _ in range(2)]
    return pts


@pytest.fixture(scope="module")
def fp64_runs(mifgpu_lib, cuda_device):
    out = {}
    for name, c in CASES.items():
        s = make(mifgpu_lib, c, mifgpu_lib.FP64)
        st = initial_state(s, c)
        r, g = loss_and_grad(s, c, st)
        out[name] = (s, st, r, g)
    return out


@pytest.mark.parametrize("name", sorted(CASES))
def test_loss_matches_final_state(fp64_runs, name):
    s, st, r, _ = fp64_runs[name]
    c = CASES[name]
    assert r["loss"] > 0
    # gradient_ke leaves the context at the final state
    assert abs(ke_numpy(s, c) - r["loss"]) <= 1e-12 * r["loss"]


@pytest.mark.parametrize("name", sorted(CASES))
def test_finite_differences_pointwise(fp64_runs, name):
    s, st, r, g = fp64_runs[name]
    c = CASES[name]
    rng = np.random.default_rng(11)
    gmax = max(np.abs(g[n]).max() for n in "uvwp")
    worst = 0.0
    for n in "uvwp":
        for pt in probe_points(st[n].shape, rng):
            plus = {k: v.copy() for k, v in st.items()}
            minus = {k: v.copy() for k, v in st.items()}
            plus[n][pt] += EPS_POINT
            minus[n][pt] -= EPS_POINT
            fd = (loss_only(s, c, plus) - loss_only(s, c, minus)) / (2 * EPS_POINT)
            adj = g[n][pt]
            # entries far below the field's largest are compared on that scale
            err = abs(fd - adj) / max(abs(adj), 1e-2 * gmax)
            worst = max(worst, err)
            assert err <= TOL, f"{name} {n}{pt}: fd {fd:.12e} adjoint {adj:.12e} rel {err:.2e}"
    print(f"{name}: worst pointwise relative error {worst:.2e}")


@pytest.mark.parametrize("name", sorted(CASES))
def test_dot_product_tangent_linear(fp64_runs, name):
    """<lambda, delta> against d/de loss(x + e delta) of the FP64 forward map."""
    s, st, r, g = fp64_runs[name]
    c = CASES[name]
    rng = np.random.default_rng(3)
    delta = {n: rng.standard_normal(st[n].shape) for n in "uvwp"}
    adj = sum(float(np.sum(g[n] * delta[n])) for n in "uvwp")
    e = EPS
    plus = {n: st[n] + e * delta[n] for n in "uvwp"}
    minus = {n: st[n] - e * delta[n] for n in "uvwp"}
    tl = (loss_only(s, c, plus) - loss_only(s, c, minus)) / (2 * e)
    err = abs(tl - adj) / abs(tl)
    print(f"{name}: dot-product test tangent-linear {tl:.15e} adjoint {adj:.15e} rel {err:.2e}")
    assert err <= TOL


@pytest.mark.parametrize("name", sorted(CASES))
def test_forcing_amplitude_derivative(fp64_runs, name):
    s, st, r, g = fp64_runs[name]
    c = CASES[name]
    a = c["alpha"]
    # alpha moves the loss by as little as 1e-6 per unit on the short wall case:
    # the larger step keeps the difference clear of the loss's last bits
    fd = (loss_only(s, c, st, a + EPS_POINT) - loss_only(s, c, st, a - EPS_POINT)) / (2 * EPS_POINT)
    err = abs(fd - r["dloss_dalpha"]) / abs(fd)
    print(f"{name}: dL/dalpha fd {fd:.12e} adjoint {r['dloss_dalpha']:.12e} rel {err:.2e}")
    assert err <= TOL


def test_checkpoint_interval_does_not_change_gradient(fp64_runs):
    s, st, r, g = fp64_runs["periodic"]
    c = CASES["periodic"]
    for every in (1, c["nsteps"]):
        r2, g2 = loss_and_grad(s, c, st, every=every)
        assert r2["loss"] == r["loss"]  # fixed-order reductions
        for n in "uvwp":
            np.testing.assert_array_equal(g2[n], g[n])
        assert r2["dloss_dalpha"] == r["dloss_dalpha"]


def test_backward_with_seeds_matches_ke(fp64_runs):
    """mifgpu_backward seeded with d KE / d u_final equals mifgpu_gradient_ke."""
    s, st, r, g = fp64_runs["dirichlet"]
    c = CASES["dirichlet"]
    s.set_forcing_amplitude(c["alpha"])
    s.load_state(st)
    s.run(c["t0"], c["nsteps"])
    vol = np.prod([c["size"][d] / (c["n_global"][d] - 1) for d in range(3)])
    x0, x1, y0, y1, z0, z1 = c["box"]
    seeds = {}
    for comp, n in enumerate("uvw"):
        a = s.download(n)
        x, y, z = coords(c, comp, a.shape)
        m = np.zeros(a.shape, bool)
        m[1:-1, 1:-1, 1:-1] = True
        m &= (x >= x0) & (x <= x1) & (y >= y0) & (y <= y1) & (z >= z0) & (z <= z1)
        seeds[n] = np.where(m, vol * a, 0.0)
    s.load_state(st)
    rb = s.backward(c["t0"], c["nsteps"], c["every"], seeds)
    for n in "uvwp":
        np.testing.assert_allclose(s.adjoint(n), g[n], rtol=0, atol=1e-13 * np.abs(g[n]).max())
    assert rb["dloss_dalpha"] == pytest.approx(r["dloss_dalpha"], rel=1e-12)


def test_fp32_adjoint_tracks_fp64(mifgpu_lib, fp64_runs):
    for name in ("periodic", "dirichlet"):
        _, st, r, g = fp64_runs[name]
        c = CASES[name]
        s32 = make(mifgpu_lib, c, mifgpu_lib.MIXED)
        r32, g32 = loss_and_grad(s32, c, st)
        s32.close()
        assert r32["loss"] == pytest.approx(r["loss"], rel=1e-5)
        for n in "uvwp":
            err = np.abs(g32[n] - g[n]).max() / np.abs(g[n]).max()
            print(f"{name} FP32 adjoint {n}: max rel error {err:.2e}")
            assert err <= 1e-4, (name, n, err)
        assert r32["dloss_dalpha"] == pytest.approx(r["dloss_dalpha"], rel=1e-4)


def test_autograd_function(mifgpu_lib, fp64_runs):
    torch = pytest.importorskip("torch")
    import mif_autograd

    s, st, r, g = fp64_runs["periodic"]
    c = CASES["periodic"]
    ins = [torch.tensor(st[n], dtype=torch.float64, requires_grad=True) for n in "uvwp"]
    alpha = torch.tensor(c["alpha"], dtype=torch.float64, requires_grad=True)
    outs = mif_autograd.ProjectionSteps.apply(s, c["t0"], c["nsteps"], c["every"], *ins, alpha)
    vol = float(np.prod([c["size"][d] / (c["n_global"][d] - 1) for d in range(3)]))
    x0, x1, y0, y1, z0, z1 = c["box"]
    loss = 0.0
    for comp, o in enumerate(outs[:3]):
        x, y, z = coords(c, comp, tuple(o.shape))
        m = np.zeros(o.shape, bool)
        m[1:-1, 1:-1, 1:-1] = True
        m &= (x >= x0) & (x <= x1) & (y >= y0) & (y <= y1) & (z >= z0) & (z <= z1)
        loss = loss + 0.5 * vol * (o[torch.from_numpy(m)] ** 2).sum()
    loss.backward()
    assert float(loss.detach()) == pytest.approx(r["loss"], rel=1e-12)
    for n, t in zip("uvwp", ins):
        np.testing.assert_allclose(t.grad.numpy(), g[n], rtol=0, atol=1e-13 * np.abs(g[n]).max())
    assert float(alpha.grad) == pytest.approx(r["dloss_dalpha"], rel=1e-12)
