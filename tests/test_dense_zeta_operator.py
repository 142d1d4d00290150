"""The dense zeta operator against the oracle's zeta derivative (CPU, no device).

ATI_OPT_DENSE_ZETA replaces the mixed path's zeta line solves by d = M f, with
one matrix M a block built on the host from the line algorithm;
ati_dense_zeta_operator exports that builder in FP64.  Here M is applied to
every zeta line of a random field and compared with the oracle's periodic
closure (mpigo with n45 = 0) and derivative along zeta
(src/Subroutines3D.f90:16-141) of the same field: equal to FP64 rounding;
and equal to the committed golden operators of periodic lines, which a second,
independent numpy restatement made.
The rows of M sum to zero, which the kernel relies on when it takes each
line's first value out before the product; zeta lines past 64 points have no
operator.
"""
import numpy as np
import pytest

from tandemproject_gb300.solver import AtiError, dense_zeta_operator


def _oracle(cfg):
    from oracle.oracle import OracleCase
    from tandemproject_gb300.grid import aerofoil_grid
    o = OracleCase(cfg)
    g = aerofoil_grid(cfg)
    for mb in range(cfg.nblocks):
        o.set_grid(mb, g[mb])
    o.init()
    return o


@pytest.mark.parametrize("lze", [12, 19, 31, 47])
def test_operator_equals_oracle_zeta_derivative(ati_lib, oracle_lib, lze):
    from tandemproject_gb300.config import small_case
    cfg = small_case(lxibk=(16, 40, 16), letbk=(12, 12), lzebk=(lze,))
    o = _oracle(cfg)
    rng = np.random.default_rng(lze)
    f = {}
    for mb in range(cfg.nblocks):
        r = np.zeros((3, o.npts(mb)))
        r[0] = 2.0 + rng.standard_normal(o.npts(mb))
        f[mb] = r[0].copy()
        o.set_field(mb, 3, r)
    o.mpigo(0, 1, 0)
    o.deriv(3, 1, 1)
    for mb in range(cfg.nblocks):
        lxi, let, lz, _ = o.dims[mb]
        M = dense_zeta_operator(cfg, mb)
        L = lz + 1
        assert M.shape == (L, L)
        lines = f[mb].reshape(L, let + 1, lxi + 1)  # zeta slowest: the points of one zeta line are a plane apart
        d_dense = np.einsum("ij,jab->iab", M, lines)
        d_orc = o.get_field(mb, 3)[2].reshape(L, let + 1, lxi + 1)
        # measured: 1.5e-15 to 2.0e-15 (13- to 48-point lines); row sums 5e-16 to 2e-15 of the largest entry
        assert np.max(np.abs(d_dense - d_orc)) <= 1e-13 * np.max(np.abs(d_orc)), mb
        assert np.max(np.abs(M.sum(axis=1))) <= 1e-14 * np.max(np.abs(M)), mb
    o.close()


def test_no_operator_past_64_points(ati_lib):
    from tandemproject_gb300.config import small_case
    with pytest.raises(AtiError):
        dense_zeta_operator(small_case(lxibk=(16, 40, 16), letbk=(12, 12), lzebk=(64,)), 0)


def test_operator_of_the_0p6m_preset(ati_lib):
    """the 20-point zeta lines of the 0.61 M-point aerofoil case: every block
    has the same operator (the same line length and periodic closure)"""
    from tandemproject_gb300.config import PRESETS
    cfg = PRESETS["naca0012_0p6m"]
    ms = [dense_zeta_operator(cfg, mb) for mb in range(cfg.nblocks)]
    assert ms[0].shape == (cfg.lzebk[0] + 1,) * 2
    for m in ms[1:]:
        assert np.array_equal(m, ms[0])


@pytest.mark.parametrize("L", [13, 20])
def test_operator_equals_the_golden_periodic_operator(ati_lib, L):
    """the committed golden operator of a periodic zeta line (tests/golden/make_golden.py: an independent numpy
    restatement, closure rows on unit vectors and numpy.linalg.solve for the left-hand side)"""
    import os
    from tandemproject_gb300.config import small_case
    gold = np.load(os.path.join(os.path.dirname(__file__), "golden", "line_operators.npz"))[f"deriv_p{L}"]
    M = dense_zeta_operator(small_case(lzebk=(L - 1,)), 0)
    assert M.shape == gold.shape
    assert np.max(np.abs(M - gold)) <= 1e-13 * np.max(np.abs(gold))  # measured 3.2e-15 (13 points), 4.1e-15 (20)
