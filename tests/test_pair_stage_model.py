"""CPU model of the two-points-per-thread stage kernel's index algebra.

`stage_pair_kernel` (csrc/stencil_impl.cuh) is the compensated Y2 / Y3 / U*
stage with the preceding projection inside. A CTA of 32 x 4 threads owns a
64 x 4 point tile from (i0, j0) = (1 + 64 bx, 1 + 4 by), each thread the pair
(i0 + 2 tx, i0 + 2 tx + 1) of row j0 + ty. It marches through its planes with
a shared-memory ring filled by TMA boxes from x = i0 - 5. This file restates,
in plain Python, the index arithmetic the kernel uses:

* the launch grid (`StageLaunch::go`, `launch_stage`);
* the interior masks of the velocity updates;
* the pressure writes: own pairs, the x = 0 / y = 0 / right-halo edge writes,
  and plane 0;
* the ring, phi and halo indices of every tap and projection;
* the TMA box origins.

Over many geometries (odd and even extents, periodic axes, one tile and
several) it checks:
* every interior point of every velocity component is updated exactly once,
  and nothing else;
* every pressure node is written exactly once on every plane;
* every shared-memory index stays inside its slot;
* every TMA box starts 16-byte aligned in x.

The GPU parity tests check the values; this model checks, with no GPU, that
the tiling covers each geometry exactly.
"""
import itertools

import pytest

# csrc/stencil_impl.cuh constants
kTX, kTY = 32, 4
kQX = 2 * kTX
kQHX = kQX + 8
kHY = kTY + 2
kQPL = kQHX * kHY
kQSlot = 448
kPhiRows = kTY + 3
kQPhiPL = kQHX * kPhiRows
kQPhiSlot = 512


def geometry(n_global, periodic):
    """Extents as mifgpu_create sets them (csrc/capi.cu)."""
    E = [n + 1 if p else n for n, p in zip(n_global, periodic)]
    Es = [E[0] if periodic[0] else E[0] + 1, E[1] + 1, E[2] + 1]
    PX = (max(Es[0], E[0]) + 7) // 8 * 8
    return dict(E=E, Es=Es, PX=PX, PY=Es[1], PZ=Es[2], periodic=periodic)


def ext(g, c, d):
    return g["Es"][d] if c == d else g["E"][d]


def cdiv(a, b):
    return (a + b - 1) // b


def launch(g, kc):
    """The pair kernel's grid and plane ranges."""
    ni = max(g["Es"][0], g["E"][0])
    nk = g["Es"][2] - 2
    grid = (cdiv(ni - 2, kQX), cdiv(g["Es"][1] - 2, kTY), cdiv(nk, kc))
    zmax = g["Es"][2] - 1
    planes = [(1 + bz * kc, min(1 + bz * kc + kc, zmax)) for bz in range(grid[2])]
    return grid, planes


def cta_writes(g, bx, by):
    """Velocity points (c, i, j) a CTA updates on an interior plane, and the
    pressure nodes (i, j) it writes, per the kernel's masks and edges."""
    E0, E1 = g["E"][0], g["E"][1]
    i0, j0 = 1 + bx * kQX, 1 + by * kTY
    grid, _ = launch(g, 4)
    vel, p = [], []
    edge_x0, edge_y0 = bx == 0, by == 0
    edge_xr = i0 + kQX == E0 - 1 and bx + 1 == grid[0]  # the last tile's right halo

    def p_edge(hx, hy):
        pi, pj = i0 - 5 + hx, j0 - 1 + hy
        if pi < E0 and pj < E1:
            p.append((pi, pj))

    for ty in range(kTY):
        for tx in range(kTX):
            i, j = i0 + 2 * tx, j0 + ty
            for x in (i, i + 1):
                for c in range(3):
                    # xy_mask: 1 <= x < ext - 1, 1 <= y < ext - 1
                    if 1 <= x < ext(g, c, 0) - 1 and 1 <= j < ext(g, c, 1) - 1:
                        vel.append((c, x, j))
                if x < E0 and j < E1:  # own_pa / own_pb
                    p.append((x, j))
            # write_p_edges
            if edge_x0 and tx == 0:
                p_edge(4, ty + 1)
            if edge_xr and tx == kTX - 1:
                p_edge(kQX + 5, ty + 1)
            if edge_y0 and ty == 0:
                p_edge(5 + 2 * tx, 0)
                p_edge(6 + 2 * tx, 0)
                if edge_x0 and tx == 0:
                    p_edge(4, 0)
                if edge_xr and tx == kTX - 1:
                    p_edge(kQX + 5, 0)
    return vel, p


GEOMETRIES = [
    # the smallest grids the library accepts
    ((3, 3, 3), (False, False, False)),
    ((4, 3, 5), (True, False, True)),
    ((3, 4, 3), (True, True, True)),
    ((5, 3, 4), (False, True, False)),
    ((9, 9, 9), (False, False, False)),
    ((17, 18, 19), (False, False, False)),
    ((26, 27, 28), (False, True, False)),
    ((33, 25, 29), (True, False, True)),
    ((32, 33, 30), (True, True, True)),
    ((65, 65, 65), (False, False, False)),
    ((64, 20, 9), (True, False, False)),   # periodic x, E0 = 65: the last node on the right halo
    ((66, 10, 7), (True, False, False)),
    ((129, 9, 6), (False, False, False)),  # 128 interior x points: two full tiles
    ((130, 11, 5), (False, True, False)),
    ((193, 6, 5), (True, True, False)),
]


@pytest.mark.parametrize("n_global,periodic", GEOMETRIES)
def test_tiles_cover_each_point_once(n_global, periodic):
    g = geometry(n_global, periodic)
    grid, planes = launch(g, 4)
    vel, p = [], []
    for bx, by in itertools.product(range(grid[0]), range(grid[1])):
        v, q = cta_writes(g, bx, by)
        vel += v
        p += q
    # velocity: each interior (x, y) of each component once (the z range is
    # the march's, checked below)
    want_vel = [(c, x, y) for c in range(3) for x in range(1, ext(g, c, 0) - 1) for y in range(1, ext(g, c, 1) - 1)]
    assert sorted(vel) == sorted(want_vel)
    # pressure: every node of the plane once
    want_p = [(x, y) for x in range(g["E"][0]) for y in range(g["E"][1])]
    assert sorted(p) == sorted(want_p)
    # planes: the marches cover 1 .. Es2 - 2 once, plane 0 by the kbeg == 1
    # CTAs; that is every pressure plane, and every interior plane of each
    # component (k < ext(c, 2) - 1, the kernel's lim_c)
    ks = [k for kb, ke in planes for k in range(kb, ke)]
    assert sorted(ks) == list(range(1, g["Es"][2] - 1))
    assert sorted([0] + ks) == list(range(g["E"][2]))
    for c in range(3):
        assert set(range(1, ext(g, c, 2) - 1)) <= set(ks)


@pytest.mark.parametrize("n_global,periodic", GEOMETRIES)
def test_ring_indices_and_tma_boxes(n_global, periodic):
    g = geometry(n_global, periodic)
    grid, _ = launch(g, 4)
    for bx in range(grid[0]):
        i0 = 1 + bx * kQX
        # TMA boxes: x = i0 - 5 (ring fields and phi) is a multiple of 4 floats
        assert (i0 - 5) * 4 % 16 == 0
    for ty in range(kTY):
        for tx in range(kTX):
            o_r = (ty + 1) * kQHX + 5 + 2 * tx
            o_p = o_r + kQHX
            assert o_r % 2 == 1 and o_p % 2 == 1
            # ring taps of the pair: x +- 1 as aligned pairs, y +- 1 rows
            for idx in (o_r - 1, o_r + 1, o_r + 2, o_r - kQHX, o_r + kQHX + 1, o_r + 1 - kQHX, o_r - 1 + kQHX):
                assert 0 <= idx < kQPL <= kQSlot
            assert (o_r - 1) % 2 == 0 and (o_r + 1) % 2 == 0 and (o_r + 1 - kQHX) % 2 == 0
            for idx in (o_p - 1, o_p + 2, o_p - kQHX, o_p - kQHX + 1):
                assert 0 <= idx < kQPhiPL <= kQPhiSlot
    # halo points of the projection: rows hy = 0 and kTY + 1 (pairs),
    # columns hx = 4 and kQX + 5 (single points)
    for tid in range(2 * kTX + 2 * (kTY + 2)):
        if tid < kTX:
            hx, hy = 5 + 2 * tid, 0
        elif tid < 2 * kTX:
            hx, hy = 5 + 2 * (tid - kTX), kTY + 1
        elif tid < 2 * kTX + kTY + 2:
            hx, hy = 4, tid - 2 * kTX
        else:
            hx, hy = kQX + 5, tid - 2 * kTX - (kTY + 2)
        h_r, h_p = hy * kQHX + hx, (hy + 1) * kQHX + hx
        pair = tid < 2 * kTX
        assert 0 <= h_r and h_r + (1 if pair else 0) < kQPL
        assert 0 <= h_p - kQHX and h_p + (2 if pair else 0) < kQPhiPL
        assert hx - 1 >= 0 and hx + (2 if pair else 0) < kQHX


def test_halo_projection_covers_the_taps():
    """Every ring point a stencil tap of an own point reads is the own pair
    or a projected halo point: rows 0 and kTY + 1 for hx = 5 .. kQX + 4, and
    the columns hx = 4 and kQX + 5 for every row."""
    projected = {(hx, hy) for hy in range(1, kTY + 1) for hx in range(5, 5 + kQX)}
    projected |= {(hx, hy) for hy in (0, kTY + 1) for hx in range(5, 5 + kQX)}
    projected |= {(hx, hy) for hx in (4, kQX + 5) for hy in range(kTY + 2)}
    # tap offsets (dx, dy) in a plane, include/MomentumEquation.h's stencils
    offsets = {(0, 0), (-1, 0), (1, 0), (0, -1), (0, 1), (-1, 1), (1, -1)}
    for ty in range(kTY):
        for tx in range(kTX):
            for hx in (5 + 2 * tx, 6 + 2 * tx):
                for dx, dy in offsets:
                    assert (hx + dx, ty + 1 + dy) in projected
