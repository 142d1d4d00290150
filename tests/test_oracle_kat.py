"""Known-answer tests that pin the CPU oracle to properties of the
reference's scheme (the reference ships no tests or golden outputs).

Each test names the reference lines whose property it checks."""
import math
import os

import numpy as np
import pytest

from conftest import ROOT


@pytest.fixture(scope="module")
def orc(oracle_lib):
    from oracle.oracle import OracleCase
    from tandemproject_gb300.config import small_case
    from tandemproject_gb300.grid import aerofoil_grid
    cfg = small_case()
    o = OracleCase(cfg)
    g = aerofoil_grid(cfg)
    for mb in range(cfg.nblocks):
        o.set_grid(mb, g[mb])
    o.init()
    o.grid = g
    return o


def block_field(o, mb, fn):
    lxi, let, lze, n = o.dims[mb]
    k, j, i = np.meshgrid(np.arange(lze + 1), np.arange(let + 1), np.arange(lxi + 1), indexing="ij")
    return fn(i, j, k).ravel().astype(np.float64)


def test_deriv_of_constant_is_exactly_zero(orc):
    """Every one-sided and interior RHS row is a difference
    (src/Subroutines3D.f90:103-123): d/dxi, d/deta of a constant are 0."""
    for mb in range(6):
        orc.set_field(mb, 3, np.full((3, orc.npts(mb)), 3.25))
    orc.mpigo(0, 1, 0)
    orc.deriv(1, 1, 1)
    for mb in range(6):
        assert np.all(orc.get_field(mb, 3)[0] == 0.0)
    for mb in range(6):
        orc.set_field(mb, 3, np.full((3, orc.npts(mb)), 3.25))
    orc.mpigo(0, 1, 0)
    orc.deriv(2, 1, 1)
    orc.deriv(3, 1, 1)
    for mb in range(6):
        r = orc.get_field(mb, 3)
        assert np.all(r[1] == 0.0)
        # periodic closure: pbci and pbco sum to zero only to round-off
        assert np.max(np.abs(r[2])) < 1e-13


def test_filter_keeps_constant(orc):
    """Filter rows are second differences, ghosts extrapolate a constant
    exactly (src/Subroutines3D.f90:166-188)."""
    for mb in range(6):
        orc.set_field(mb, 3, np.full((3, orc.npts(mb)), -1.5))
    orc.mpigo(1, 1, 0)
    orc.filte(1, 1)
    orc.filte(2, 1)
    for mb in range(6):
        assert np.all(orc.get_field(mb, 3)[0] == -1.5)
    orc.filte(3, 1)
    for mb in range(6):
        assert np.max(np.abs(orc.get_field(mb, 3)[0] + 1.5)) < 1e-14


def test_filter_removes_grid_scale_mode(orc):
    """The interior filter (fcint, src/Subroutineso.f90:91-103) has a zero
    of its transfer function at the grid scale pi: (-1)^i is removed away
    from the line ends.  The one-sided end rows leave the mode at the ends and
    their influence decays by about 0.75 per point, so only the centre of the
    65-point line is checked (a filter passing the mode would leave 1.0)."""
    mb = 1  # 65 points along xi
    f = block_field(orc, mb, lambda i, j, k: (-1.0) ** i)
    r = np.zeros((3, orc.npts(mb)))
    r[0] = f
    for b in range(6):
        orc.set_field(b, 3, r if b == mb else np.zeros((3, orc.npts(b))))
    orc.mpigo(1, 1, 0)
    orc.filte(1, 1)
    lxi, let, lze, _ = orc.dims[mb]
    out = orc.get_field(mb, 3)[0].reshape(lze + 1, let + 1, lxi + 1)
    assert np.max(np.abs(out[:, :, 30:35])) < 1e-4


def test_interior_modified_wavenumber(orc):
    """Interior derivative of sin(k i) equals the scheme's modified
    wavenumber times cos(k i) (alpha, beta, aa, ab, ac at
    src/MainVar3D.f90:34-38), far from the line ends."""
    al, be = 0.5862704032801503, 0.09549533555017055
    aa, ab, ac = 0.6431406736919156, 0.2586011023495066, 0.007140953479797375
    mb = 1
    for kw in (0.3, 0.9, 1.6):
        f = block_field(orc, mb, lambda i, j, k: np.sin(kw * i))
        r = np.zeros((3, orc.npts(mb)))
        r[0] = f
        for b in range(6):
            orc.set_field(b, 3, r if b == mb else np.zeros((3, orc.npts(b))))
        orc.mpigo(0, 1, 0)
        orc.deriv(1, 1, 1)
        lxi, let, lze, _ = orc.dims[mb]
        out = orc.get_field(mb, 3)[0].reshape(lze + 1, let + 1, lxi + 1)
        kmod = (2 * aa * math.sin(kw) + 2 * ab * math.sin(2 * kw) + 2 * ac * math.sin(3 * kw)) / (
            1 + 2 * al * math.cos(kw) + 2 * be * math.cos(2 * kw))
        i = np.arange(28, 37)
        # the one-sided boundary rows' influence decays into the interior; at the
        # centre it stays an order of magnitude below the gap between the
        # scheme's modified wavenumber and the exact one, which the test resolves
        err = np.max(np.abs(out[3, 5, 28:37] - kmod * np.cos(kw * i)))
        assert err < 0.1 * abs(kmod - kw), (kw, err, kmod - kw)


def test_penta_lu_reproduces_matrix(orc):
    """L*U of penta's factors (src/Subroutineso.f90:15-67) is the
    pentadiagonal matrix with the one-sided boundary rows
    (src/Main3D.f90:295-297)."""
    albed = orc.scheme(2, 30).reshape(2, 3, 5)
    for nn, filt in ((1, 0), (2, 0)):
        u, l = orc.factors(0, nn, filt)
        n = u.shape[1]
        Lm = np.eye(n)
        Um = np.zeros((n, n))
        for i in range(n):
            if i >= 1:
                Lm[i, i - 1] = l[1, i]
            if i >= 2:
                Lm[i, i - 2] = l[0, i]
            Um[i, i] = 1.0 / u[0, i]
            if i + 1 < n:
                Um[i, i + 1] = u[1, i] / u[0, i]
            if i + 2 < n:
                Um[i, i + 2] = u[2, i] / u[0, i]
        A = Lm @ Um
        E = np.zeros((n, n))
        al, be = 0.5862704032801503, 0.09549533555017055
        for i in range(n):
            if i < 3:
                for o in range(-2, 3):
                    if 0 <= i + o < n:
                        E[i, i + o] = albed[0, i, o + 2]
            elif i > n - 4:
                for o in range(-2, 3):
                    if 0 <= i - o < n:
                        E[i, i - o] = albed[0, n - 1 - i, o + 2]
            else:
                E[i, i - 2:i + 3] = [be, al, 1, al, be]
        assert np.max(np.abs(A - E)) < 1e-13


def test_periodic_coordinate_derivative(orc):
    """With n45 = 1 the periodic closure re-bases the spanwise coordinate
    jump (src/Subroutines3D.f90:59-78), so dz/dzeta is the uniform spacing
    -span/lze at every point, ends included."""
    for mb in range(6):
        r = np.zeros((3, orc.npts(mb)))
        r[0] = orc.grid[mb][2].ravel()
        orc.set_field(mb, 3, r)
    orc.mpigo(0, 1, 1)
    orc.deriv(3, 1, 1)
    span, lze = 0.1, 12
    for mb in range(6):
        assert np.max(np.abs(orc.get_field(mb, 3)[2] + span / lze)) < 1e-14


def test_dt_ramp_starts_at_zero(oracle_lib):
    """dt = dts + (dte-dts) sin^2(0.05 pi (n-ndt)) gives dt = 0 for n = 0, 1
    from a fresh start (src/Main3D.f90:521, 588-610)."""
    from oracle.oracle import OracleCase
    from tandemproject_gb300.config import small_case
    from tandemproject_gb300.grid import aerofoil_grid
    cfg = small_case(lxibk=(48, 120, 48), letbk=(39, 39), lzebk=(12,))
    o = OracleCase(cfg)
    g = aerofoil_grid(cfg)
    for mb in range(6):
        o.set_grid(mb, g[mb])
    o.init()
    q0 = [o.get_state(mb).copy() for mb in range(6)]
    o.step(1)
    assert o.get_time()[2] == 0.0
    o.step(1)
    n, ndt, dt, dts, dte, timo = o.get_time()
    assert (n, ndt, dt, timo) == (2, 1, 0.0, 0.0) and dte > 0.0
    o.step(1)
    assert o.get_time()[2] > 0.0
    # the first steps moved the state only through filter, wall and averaging
    assert all(np.all(np.isfinite(o.get_state(mb))) for mb in range(6))
    assert any(not np.array_equal(q0[mb], o.get_state(mb)) for mb in range(6))
