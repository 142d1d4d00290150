"""Host-side helpers of the batched and serving workloads
(tandemproject_gb300.workloads) on the CPU: the sizing rule, the grid
relaxation used when a grid folds, and the fold-free grid search; and the
named presets' sizes."""
import numpy as np
import pytest

from tandemproject_gb300.workloads import relax, sized_case, valid_grid


FLOOR = 6 * 160 * 56 * 16  # the smallest case: the in-plane minimum and 16 spanwise points


@pytest.mark.parametrize("npts,nz", [(0.5e6, 16), (2.0e6, 24), (6.0e6, 40), (20.0e6, 48)])
def test_sized_case_hits_its_point_count(npts, nz):
    cfg = sized_case(npts, nz, np.random.default_rng(0))
    nx, ny, nzz = cfg.lxibk[0] + 1, cfg.letbk[0] + 1, cfg.lzebk[0] + 1
    assert nx >= 160 and ny >= 56 and 16 <= nzz <= 48
    want = max(npts, FLOOR)  # below the floor a case keeps the minimum in-plane grid
    assert abs(cfg.npoints - want) / want < 0.15, (cfg.npoints, npts)
    assert 0.002 <= cfg.smgrid <= 0.0075
    assert cfg.nsmf == 0 and cfg.timf == 1.0  # the deck's smooth start over one time unit


def test_relax_adds_eta_lines_at_about_the_same_size():
    cfg = sized_case(3.0e6, 24, np.random.default_rng(0))
    r = relax(cfg)
    assert all(b + 1 == round((a + 1) * 1.25) for a, b in zip(cfg.letbk, r.letbk))
    assert all(b < a for a, b in zip(cfg.lxibk, r.lxibk))
    assert abs(r.npoints - cfg.npoints) / cfg.npoints < 0.05
    assert r.lzebk == cfg.lzebk and 0.002 <= r.smgrid <= 0.0075


def test_valid_grid_is_fold_free():
    from tandemproject_gb300.grid import min_cell_jacobian
    cfg, g = valid_grid(sized_case(0.5e6, 16, np.random.default_rng(0), thick=18.0))
    j = min_cell_jacobian(g)
    assert len(g) == cfg.nblocks
    assert all(a < 0 and b < 0 for a, b in j) or all(a > 0 and b > 0 for a, b in j), j


@pytest.mark.parametrize("name,points,precision", [
    ("naca0012_0p2m", 227_760, 0), ("naca0012_0p6m", 612_800, 0), ("naca0012_3p5m", 3_538_944, 0),
    ("naca0012_8p8m", 8_847_360, 0), ("naca0012_25m", 24_576_000, 1)])
def test_presets_are_the_named_workloads(name, points, precision):
    from tandemproject_gb300.config import PRESETS
    cfg = PRESETS[name]
    assert cfg.npoints == points and cfg.precision == precision and cfg.nblocks == 6
