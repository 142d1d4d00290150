"""Dense zeta derivatives of the mixed path (k_sweep_dense, ATI_OPT_DENSE_ZETA).

On blocks whose zeta faces are periodic onto the block itself, the zeta
derivative of a line is a fixed linear map of its values: the host builds the
L x L operator of every block in FP64 from the line algorithm (closures,
end rows, interior stencil, LU solve; src/Subroutines3D.f90:84-141) and the
kernel forms the product in FP32.  Its rounding differs from the recurrence's,
so the checks are against the FP64 path: after a few steps the dense run's
error per conserved variable stays within a small factor of the recurrence's.
The kernel comes in widths of 16, 24, 32, 48 and 64 points (the cases take
the 16-, 24-, 32-, 48- and 64-wide ones); longer lines and the FP64 path leave
the option off.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _err(run, ref, nblocks):
    num, den = np.zeros(5), np.zeros(5)
    for mb in range(nblocks):
        q, qd = run.get_state(mb), ref.get_state(mb)
        num += np.sum((q - qd) ** 2, axis=1)
        den += np.sum(qd ** 2, axis=1)
    return np.sqrt(num / den)


@pytest.mark.parametrize("lze", [12, 23, 31, 47, 63])
def test_dense_zeta_against_fp64(ati_lib, lze):
    from tandemproject_gb300.config import FP64, MIXED, small_case
    from tandemproject_gb300.grid import aerofoil_grid
    from tandemproject_gb300.solver import setup_case
    cfg = small_case(lxibk=(31, 63, 31), letbk=(15, 15), lzebk=(lze,), precision=MIXED)
    grid = aerofoil_grid(cfg)
    ref = setup_case(cfg.replace(precision=FP64), grid=grid)
    seg = setup_case(cfg, grid=grid)
    dense = setup_case(cfg, grid=grid)
    assert not ref.set_options(dense_zeta=True)["dense_zeta"]  # the FP64 path has no dense operators
    assert not seg.set_options(dense_zeta=False)["dense_zeta"]
    assert dense.set_options(dense_zeta=True)["dense_zeta"]
    for c in (ref, seg, dense):
        c.step(20)
    e_seg, e_dense = _err(seg, ref, cfg.nblocks), _err(dense, ref, cfg.nblocks)
    assert np.all(e_seg[[0, 4]] < 1e-6), e_seg  # density and energy; the small w momentum has the largest error
    assert np.all(e_dense <= 3.0 * e_seg + 1e-9), (e_dense, e_seg)
    # the option took effect: the dense products round differently from the recurrence
    assert any(not np.array_equal(dense.get_state(mb), seg.get_state(mb)) for mb in range(cfg.nblocks))
    for c in (ref, seg, dense):
        c.close()


def test_dense_zeta_not_taken_past_64_points(ati_lib):
    from tandemproject_gb300.config import MIXED, small_case
    from tandemproject_gb300.solver import setup_case
    cfg = small_case(lxibk=(31, 63, 31), letbk=(15, 15), lzebk=(64,), precision=MIXED)
    a = setup_case(cfg)
    assert not a.set_options(dense_zeta=True)["dense_zeta"]
    a.close()


def test_dense_zeta_off_is_the_recurrence(ati_lib):
    """switching the option on and off again leaves the recurrence's results bit-identical"""
    from tandemproject_gb300.config import MIXED, small_case
    from tandemproject_gb300.solver import setup_case
    cfg = small_case(lxibk=(31, 63, 31), letbk=(15, 15), lzebk=(23,), precision=MIXED)
    a = setup_case(cfg)
    b = setup_case(cfg)
    assert a.set_options(dense_zeta=True)["dense_zeta"]
    assert not a.set_options(dense_zeta=False)["dense_zeta"]
    a.step(6)
    b.step(6)
    for mb in range(cfg.nblocks):
        assert np.array_equal(a.get_state(mb), b.get_state(mb)), mb
    a.close()
    b.close()


def test_dense_zeta_in_a_batch(ati_lib):
    """a batch of cases of different zeta line lengths (13 and 48 points): each block its own operator"""
    from tandemproject_gb300.config import FP64, MIXED, small_case
    from tandemproject_gb300.solver import setup_batch
    cfgs = [small_case(precision=MIXED), small_case(lxibk=(31, 63, 31), letbk=(15, 15), lzebk=(47,), precision=MIXED)]
    ref = setup_batch([c.replace(precision=FP64) for c in cfgs])
    seg = setup_batch(cfgs)
    dense = setup_batch(cfgs)
    assert dense.set_options(dense_zeta=True)["dense_zeta"]
    for c in (ref, seg, dense):
        c.step(10)
    nb = sum(c.nblocks for c in cfgs)
    e_seg, e_dense = _err(seg, ref, nb), _err(dense, ref, nb)
    assert np.all(e_dense <= 3.0 * e_seg + 1e-9), (e_dense, e_seg)
    assert any(not np.array_equal(dense.get_state(b), seg.get_state(b)) for b in range(nb))
    for c in (ref, seg, dense):
        c.close()
