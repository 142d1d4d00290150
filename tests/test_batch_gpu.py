"""Batched cases (ati_create_batch): several independent aerofoil cases in one
handle, one launch per kernel and one CUDA graph per step for all of them.
Each case of a batch must evolve exactly as it does alone."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def cases(precision):
    from tandemproject_gb300.config import small_case
    return [
        small_case(lxibk=(48, 120, 48), letbk=(39, 39), lzebk=(12,), precision=precision),
        small_case(lxibk=(32, 96, 32), letbk=(31, 31), lzebk=(12,), mach=0.3, aoa_deg=4.0, precision=precision),
        small_case(lxibk=(40, 100, 40), letbk=(35, 35), lzebk=(16,), mach=0.2, reoo=2e5, precision=precision),
    ]


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_batch_matches_cases_alone(ati_lib, precision):
    from tandemproject_gb300.solver import setup_batch, setup_case
    cfgs = cases(precision)
    b = setup_batch(cfgs)
    b.step(14)
    for cs, cfg in enumerate(cfgs):
        a = setup_case(cfg)
        a.step(14)
        assert b.case_time(cs) == a.get_time()
        for mb, q in enumerate(b.case_state(cs)):
            np.testing.assert_array_equal(q, a.get_state(mb))
        np.testing.assert_array_equal(b.case_forces(cs), a.forces())
        a.close()
    b.close()


def test_batch_rejects_mixed_numerics(ati_lib):
    from tandemproject_gb300.config import small_case
    from tandemproject_gb300.solver import AtiError, Batch
    with pytest.raises(AtiError):
        Batch([small_case(), small_case(fltk=0.9)])


def test_batch_cases_have_own_dt(ati_lib):
    from tandemproject_gb300.solver import setup_batch
    b = setup_batch(cases(0))
    b.step(12)
    dts = [b.case_time(cs)[2] for cs in range(b.ncase)]
    assert len(set(dts)) == 3 and all(d > 0 for d in dts)
    b.close()


def test_jacobian_sign_check(ati_lib):
    """ati_jacobian_sign: one sign per block on a good grid; the wake-line cells
    of a coarse-eta grid fold under the compact metrics and are reported."""
    from tandemproject_gb300.config import PRESETS
    from tandemproject_gb300.solver import setup_case
    from tandemproject_gb300.workloads import batch_cases, fold_free_case, valid_grid
    c = setup_case(PRESETS["naca0012_0p2m"])
    assert c.folded_blocks() == [] and len(set(c.jacobian_sign())) == 1
    c.close()
    coarse = batch_cases(16, seed=7)[5][0].replace(lxibk=(109,) * 3, letbk=(34, 34), lzebk=(45,), smgrid=0.0075)
    cfg, g = valid_grid(coarse)
    c = setup_case(cfg, grid=g)
    assert c.folded_blocks() == [2]
    c.close()
    cfg, g, c = fold_free_case(coarse)
    assert c.folded_blocks() == [] and cfg.letbk[0] > coarse.letbk[0]
    c.close()


def test_autotuned_tiles_are_candidates(ati_lib):
    from tandemproject_gb300.config import PRESETS
    from tandemproject_gb300.solver import setup_case
    c = setup_case(PRESETS["naca0012_0p2m"])
    xi, s2, s3, pt = c.tiles()
    assert xi == 64 and s2 in (32, 64, 128, 256) and s3 in (32, 64, 128, 256) and pt in (256, 1024, 4096)
    c.close()


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_pinned_tiles_give_identical_states(ati_lib, precision):
    """Tile shapes (and with them the shared-memory or global forward values of
    the eta/zeta sweeps) change timings only: states agree bit for bit."""
    from tandemproject_gb300.config import small_case
    from tandemproject_gb300.solver import AtiError, setup_case
    cfg = small_case(lxibk=(48, 120, 48), letbk=(39, 39), lzebk=(12,), precision=precision)
    a, b, c = setup_case(cfg), setup_case(cfg), setup_case(cfg)  # c: the timed tiles, one size per pointwise kernel
    a.set_tiles(eta=32, zeta=256, points=256)
    b.set_tiles(eta=256, zeta=32, points=4096)
    assert a.tiles() == (64, 32, 256, 256) and b.tiles() == (64, 256, 32, 4096)
    for h in (a, b, c):
        h.step(6)
    for mb in range(6):
        np.testing.assert_array_equal(a.get_state(mb), b.get_state(mb))
        np.testing.assert_array_equal(a.get_state(mb), c.get_state(mb))
    c.close()
    with pytest.raises(AtiError):
        a.set_tiles(eta=48)
    with pytest.raises(AtiError):
        a.set_tiles(points=300)
    a.close()
    b.close()


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_tile_plan_reused_without_timing(ati_lib, precision):
    """A handle set up without the tile timing (ati_set_tuning(h, 0)) takes an
    earlier handle's whole tile plan, each pointwise kernel's size included,
    and steps bit for bit as it does; a plan with a size that was not timed is
    refused."""
    from tandemproject_gb300.config import small_case
    from tandemproject_gb300.grid import aerofoil_grid
    from tandemproject_gb300.solver import AtiError, Case, setup_case
    cfg = small_case(lxibk=(48, 120, 48), letbk=(39, 39), lzebk=(12,), precision=precision)
    g = aerofoil_grid(cfg)
    a = setup_case(cfg, grid=g)
    plan = a.tile_plan()
    assert len(plan) == 11 and plan[:4] == a.tiles()
    assert all(v in (0, 256, 1024, 4096) for v in plan[4:])
    b = Case(cfg)
    b.set_tuning(False)
    for mb in range(cfg.nblocks):
        b.set_grid(mb, g[mb])
    b.init()
    b.set_tile_plan(plan)
    assert b.tile_plan() == plan
    a.step(6)
    b.step(6)
    for mb in range(cfg.nblocks):
        np.testing.assert_array_equal(a.get_state(mb), b.get_state(mb))
    bad = list(plan)
    bad[4] = 512
    with pytest.raises(AtiError):
        b.set_tile_plan(bad)
    a.close()
    b.close()
