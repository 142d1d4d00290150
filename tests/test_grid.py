"""Known-answer tests of the six-block aerofoil grid generator (grid.py), the
numpy restatement of gridaerofoil (src/Grid.f90:62-482) with gridf
(src/Subroutineso.f90:288-314), hermite2D (src/Grid.f90:485-583) and naca
(src/Grid.f90:696-711).  Every GPU and oracle test consumes these grids, so a
grid bug would otherwise pass every parity test unseen.  The expected values
are derived from the reference's formulas, not from the code under test.
"""
import math

import numpy as np
import pytest

from tandemproject_gb300.config import PRESETS, small_case
from tandemproject_gb300.grid import aerofoil_grid, gridf, min_cell_jacobian, naca

# the NACA polynomial of src/Grid.f90:702-707 with its default-real (float32) coefficients
A = [np.float32(v) for v in (0.298222773, 0.127125232, 0.357907906, 0.291984971, 0.105174606)]
K = np.float32(0.991148635)


def naca_by_hand(xc, t_percent):
    t = t_percent * float(np.float32(0.01))  # t0 * 0.01e0: a double times a default-real literal
    poly = (float(A[0]) * math.sqrt(xc) - float(A[1]) * xc - float(A[2]) * xc ** 2 + float(A[3]) * xc ** 3
            - float(A[4]) * xc ** 4)
    return t * float(K) / float(np.float32(0.2)) * poly


@pytest.mark.parametrize("xc", [0.0, 0.01, 0.1, 0.3, 0.5, 0.9, 1.0])
@pytest.mark.parametrize("t", [8.0, 12.0, 18.0])
def test_naca_half_thickness(xc, t):
    """naca(x, c, t, n): upper (n = 1) positive, lower (n = 0) its mirror image."""
    up, lo = naca(xc, 1.0, t, 1), naca(xc, 1.0, t, 0)
    assert up == pytest.approx(naca_by_hand(xc, t), rel=1e-12, abs=1e-15)
    assert lo == -up
    # chord scaling: y(x c, c) = c y(x, 1)
    assert naca(xc * 2.5, 2.5, t, 1) == pytest.approx(2.5 * up, rel=1e-12, abs=1e-15)


def test_naca_0012_shape():
    """Leading edge at 0, trailing edge closed (to the float32 rounding of the
    coefficients, whose sum is 0), maximum thickness 11.897 % of chord near
    x/c = 0.297 for t = 12."""
    assert naca(0.0, 1.0, 12.0, 1) == 0.0
    assert abs(naca(1.0, 1.0, 12.0, 1)) < 2e-8
    x = np.linspace(0.0, 1.0, 20001)
    y = np.array([naca(v, 1.0, 12.0, 1) for v in x])
    assert 2 * y.max() == pytest.approx(0.118972, abs=2e-6)
    assert x[y.argmax()] == pytest.approx(0.297, abs=2e-3)
    assert np.all(y[1:-1] > 0)


@pytest.mark.parametrize("dxo,dxn", [(0.01, 0.05), (1e-6, 0.02), (0.03, 1e-6)])
def test_gridf_quintic_end_conditions(dxo, dxn):
    """gridf is the quintic with the given end values and end slopes (per
    index) and zero second derivative at both ends; SML (1e-6) at one end
    means 'free': that end's slope becomes 2 (xn - xo)/m minus the other."""
    m, xo, xn = 40, -1.5, 2.0
    x, xxi = np.zeros(m + 1), np.zeros(m + 1)
    gridf(x, xxi, xo, xn, dxo, dxn, m, 0)
    a = dxo if dxo != 1e-6 else 2 * (xn - xo) / m - dxn
    b = dxn if dxn != 1e-6 else 2 * (xn - xo) / m - dxo
    assert x[0] == pytest.approx(xo, abs=1e-14) and x[m] == pytest.approx(xn, abs=1e-13)
    assert xxi[0] == pytest.approx(a, rel=1e-12) and xxi[m] == pytest.approx(b, rel=1e-12)
    # the polynomial itself: x(s) = aa s^5 + bb s^4 + cc s^3 + dd s + xo at s = i/m
    s = np.arange(m + 1) / m
    dl = xn - xo
    aa, bb = 6 * dl - 3 * m * (a + b), -15 * dl + m * (8 * a + 7 * b)
    cc, dd = 10 * dl - m * (6 * a + 4 * b), m * a
    assert np.allclose(x, aa * s ** 5 + bb * s ** 4 + cc * s ** 3 + dd * s + xo, rtol=0, atol=1e-13)
    # ... whose curvature vanishes at both ends (no s^2 term; 20 aa + 12 bb + 6 cc = 0)
    assert abs(20 * aa + 12 * bb + 6 * cc) < 1e-12 * (abs(aa) + abs(bb) + abs(cc))


@pytest.fixture(scope="module")
def grid06():
    cfg = PRESETS["naca0012_0p6m"]
    return cfg, aerofoil_grid(cfg)


def test_block_shapes(grid06):
    cfg, g = grid06
    assert len(g) == 6
    for mb, b in enumerate(g):
        lxi, let, lze = cfg.lxibk[mb % 3], cfg.letbk[mb // 3], cfg.lzebk[0]
        assert b.shape == (3, lze + 1, let + 1, lxi + 1)


def test_aerofoil_surface(grid06):
    """The wall rows carry the 201 surface points of the aerofoil (lxi = 200 in
    the middle blocks): block 1's top row is the lower surface, block 4's
    bottom row the upper one, both from the leading edge (-c/2, 0) to the
    trailing edge (c/2, 0), every point on the NACA 0012 curve, the two
    surfaces mirror images (0 deg incidence), and the first 25 points spaced at
    the arc length shs1 = ximod * smgrid (src/Grid.f90:305-314)."""
    cfg, g = grid06
    lo_x, lo_y = g[1][0, 0, -1, :], g[1][1, 0, -1, :]
    up_x, up_y = g[4][0, 0, 0, :], g[4][1, 0, 0, :]
    assert lo_x.size == 201 and up_x.size == 201
    for x, y in ((lo_x, lo_y), (up_x, up_y)):
        assert x[0] == -0.5 and abs(y[0]) < 1e-15
        assert x[-1] == 0.5 and abs(y[-1]) < 1e-15
        assert np.all(np.diff(x) > 0)
    assert np.array_equal(lo_x, up_x)
    assert np.max(np.abs(lo_y + up_y)) < 1e-15
    # points 26..199 take y = naca(x) at their final x; points 1..25 come from the arc-length iteration, whose last
    # step moves x by under 2^-8 * 1e-6 * shs1 after y was taken (the reference's order)
    res = [abs(up_y[i] - naca(up_x[i] + 0.5, 1.0, 12.0, 1)) for i in range(1, 200)]
    assert max(res[25:]) < 1e-15 and max(res[:25]) < 1e-9
    assert np.all(up_y[1:-1] > 0) and np.all(lo_y[1:-1] < 0)
    shs1 = cfg.ximod * cfg.smgrid
    ds = np.hypot(np.diff(up_x), np.diff(up_y))[:25]
    assert np.allclose(ds, shs1, rtol=2e-6, atol=0)
    # the thickest point: 11.897 % of chord
    assert 2 * up_y.max() == pytest.approx(0.118972, abs=2e-5)


def test_interfaces_coincide(grid06):
    """Interface points are duplicated per block (src/Grid.f90:168): the xi
    interfaces are the same points bit for bit, the eta interfaces to the
    rounding of the Hermite patches."""
    _, g = grid06
    for j in range(2):
        for i in range(2):
            a, b = g[3 * j + i], g[3 * j + i + 1]
            assert np.array_equal(a[:, :, :, -1], b[:, :, :, 0])
    for i in (0, 2):  # (blocks 1 and 4 are parted by the aerofoil: their rows are the two surfaces)
        a, b = g[i], g[i + 3]
        assert np.max(np.abs(a[:, :, -1, :] - b[:, :, 0, :])) < 1e-13


def test_spanwise_extrusion(grid06):
    """z runs from +span/2 (k = 0) to -span/2 (k = lze) in equal steps; the
    end planes are the periodic pair; x and y do not depend on k."""
    cfg, g = grid06
    lze = cfg.lzebk[0]
    for b in g:
        z = b[2, :, 0, 0]
        assert z[0] == pytest.approx(cfg.span / 2) and z[-1] == pytest.approx(-cfg.span / 2)
        assert np.allclose(np.diff(z), -cfg.span / lze, rtol=1e-12)
        assert np.all(b[2] == z[:, None, None])
        assert np.all(b[0] == b[0, :1]) and np.all(b[1] == b[1, :1])


def test_domain_extent(grid06):
    """Inflow at -0.7 domlen, lower boundary -0.7 domlen, outflow c/2 + domlen +
    szxt and upper boundary domlen + szxt (dlth, src/Grid.f90:81-82)."""
    cfg, g = grid06
    xs = np.concatenate([b[0].ravel() for b in g])
    ys = np.concatenate([b[1].ravel() for b in g])
    lo = -float(np.float32(0.7)) * cfg.domlen
    assert xs.min() == pytest.approx(lo, rel=1e-12) and ys.min() == pytest.approx(lo, rel=1e-12)
    assert xs.max() == pytest.approx(0.5 * cfg.chord + cfg.domlen + cfg.szxt, rel=1e-12)
    assert ys.max() == pytest.approx(cfg.domlen + cfg.szxt, rel=1e-12)


@pytest.mark.parametrize("preset", ["naca0012_0p2m", "naca0012_0p6m", "naca0012_3p5m"])
def test_no_folded_cells(preset):
    """Every block keeps one cell orientation (no folded cells)."""
    g = aerofoil_grid(PRESETS[preset])
    for lo, hi in min_cell_jacobian(g):
        assert lo * hi > 0 and (lo > 0) == (hi > 0)


@pytest.mark.parametrize("t", [8.0, 18.0])
def test_thickness_parameter(t):
    """The NACA 00tt thickness is a parameter (the reference fixes thk = 21,
    src/Grid.f90:75): the surface scales with it."""
    cfg = small_case(thick=t)
    g = aerofoil_grid(cfg)
    x, y = g[4][0, 0, 0, :], g[4][1, 0, 0, :]
    for i in range(26, x.size - 1):
        assert y[i] == pytest.approx(naca(x[i] + 0.5, 1.0, t, 1), abs=1e-15)
    for i in range(1, 26):
        assert y[i] == pytest.approx(naca(x[i] + 0.5, 1.0, t, 1), abs=1e-9)
    assert 2 * y.max() == pytest.approx(0.118972 * t / 12.0, rel=5e-3)
