"""TMA staging of the mixed path's segmented eta and zeta derivative sweeps.

Each tile of 32 lines comes into shared memory as one tensor copy
(cp.async.bulk.tensor) when the blocks' FP32 planes can be described by a
tensor map (bases and row or plane sizes multiples of 16 bytes, lines of at
most 256 points), else by per-thread asynchronous copies.  The staged values
are the same either way, so the results must be bit-identical.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _aligned_case(**kw):
    from tandemproject_gb300.config import MIXED, small_case
    # 6 blocks of 32/64/32 x 16 x 16 points: every row and plane a multiple of 4 floats
    return small_case(lxibk=(31, 63, 31), letbk=(15, 15), lzebk=(15,), precision=MIXED, **kw)


def test_tma_staging_bit_identical_to_async_copies(ati_lib):
    from tandemproject_gb300.solver import setup_case
    cfg = _aligned_case()
    a = setup_case(cfg)
    b = setup_case(cfg)
    on = a.set_options(tma=True)
    assert on["tma_eta"] and on["tma_zeta"]
    off = b.set_options(tma=False)
    assert not off["tma_eta"] and not off["tma_zeta"]
    a.step(12)
    b.step(12)
    for mb in range(cfg.nblocks):
        assert np.array_equal(a.get_state(mb), b.get_state(mb)), mb
    # switching on a running case captures its step graph again and keeps going
    b.set_options(tma=True)
    a.step(3)
    b.step(3)
    for mb in range(cfg.nblocks):
        assert np.array_equal(a.get_state(mb), b.get_state(mb)), mb
    a.close()
    b.close()


def test_tma_off_where_geometry_does_not_allow(ati_lib):
    """Rows of 25 or 65 floats are not multiples of 16 bytes: eta stays on
    per-thread copies; the zeta planes (25 x 17 = 425 points) too."""
    from tandemproject_gb300.config import MIXED, small_case
    from tandemproject_gb300.solver import setup_case
    c = setup_case(small_case(precision=MIXED))
    o = c.set_options(tma=True)
    assert not o["tma_eta"] and not o["tma_zeta"]
    c.step(3)
    c.close()


def test_tma_on_the_large_presets(ati_lib):
    """The 8.85 M and 24.6 M-point cases (rows of 384 and 640 points) stage by TMA in both directions."""
    from tandemproject_gb300.config import MIXED, PRESETS
    from tandemproject_gb300.solver import Case
    for name in ("naca0012_8p8m", "naca0012_25m"):
        c = Case(PRESETS[name].replace(precision=MIXED))
        o = c.set_options(tma=True)
        assert o["tma_eta"] and o["tma_zeta"], name
        c.close()
