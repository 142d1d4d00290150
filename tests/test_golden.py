"""The oracle against tests/golden/line_operators.npz: an independent numpy
restatement of the line operators (tests/golden/make_golden.py) — sbcco with
numpy.linalg.inv, deriv/filte right-hand sides evaluated on unit vectors and
the pentadiagonal left-hand side solved with LAPACK."""
import os

import numpy as np
import pytest

from conftest import ROOT

GOLD = os.path.join(ROOT, "tests", "golden", "line_operators.npz")


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


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
    return o


def test_closure_coefficients(orc, gold):
    pbci = orc.scheme(0, 48).reshape(2, 2, 12)
    pbco = orc.scheme(1, 48).reshape(2, 2, 12)
    assert np.max(np.abs(pbci - gold["pbci"])) < 1e-12 * np.max(np.abs(gold["pbci"]))
    assert np.max(np.abs(pbco - gold["pbco"])) < 1e-12 * np.max(np.abs(gold["pbco"]))


def lines(orc, mb, nn, field):
    lxi, let, lze, _ = orc.dims[mb]
    a = field.reshape(lze + 1, let + 1, lxi + 1)
    if nn == 1:
        return a.reshape(-1, lxi + 1)
    if nn == 2:
        return np.moveaxis(a, 1, 2).reshape(-1, let + 1)
    return np.moveaxis(a, 0, 2).reshape(-1, lze + 1)


@pytest.mark.parametrize("nn", [1, 2, 3])
def test_deriv_and_filter_match_dense_operators(orc, gold, nn):
    rng = np.random.default_rng(11 + nn)
    fields = {}
    for mb in range(6):
        r = rng.standard_normal((3, orc.npts(mb)))
        fields[mb] = r
        orc.set_field(mb, 3, r)
    orc.mpigo(0, 1, 0)
    orc.deriv(nn, 1, 1)
    for mb in range(6):
        L = {1: orc.dims[mb][0], 2: orc.dims[mb][1], 3: orc.dims[mb][2]}[nn] + 1
        tag = f"{'p' if nn == 3 else 'o'}{L}"
        D = gold[f"deriv_{tag}"]
        f = lines(orc, mb, nn, fields[mb][0])
        got = lines(orc, mb, nn, orc.get_field(mb, 3)[nn - 1])
        exp = f @ D.T
        assert np.max(np.abs(got - exp)) < 1e-12 * np.max(np.abs(exp)), (mb, nn)
    for mb in range(6):
        orc.set_field(mb, 3, fields[mb])
    orc.mpigo(1, 1, 0)
    orc.filte(nn, 1)
    for mb in range(6):
        L = {1: orc.dims[mb][0], 2: orc.dims[mb][1], 3: orc.dims[mb][2]}[nn] + 1
        tag = f"{'p' if nn == 3 else 'o'}{L}"
        G = gold[f"filter_{tag}"]
        f = lines(orc, mb, nn, fields[mb][0])
        got = lines(orc, mb, nn, orc.get_field(mb, 3)[0])
        exp = f @ G.T
        assert np.max(np.abs(got - exp)) < 1e-12 * np.max(np.abs(exp)), (mb, nn)
