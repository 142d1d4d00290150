"""Outputs and on-disk formats: Cp (getCp, src/rptPost.f90:1456-1465), the
surface-pressure recorder, restart files (wrRsta/rdRsta, src/rpt.f90:555-668)
and Plot3D files (wrP3dG/wrP3dS, src/rpt.f90:115-330)."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def case(ati_lib):
    from tandemproject_gb300.config import small_case
    from tandemproject_gb300.solver import setup_case
    c = setup_case(small_case(lxibk=(48, 120, 48), letbk=(39, 39), lzebk=(12,)))
    c.step(6)
    yield c
    c.close()


def pressure(q, gamm1=1.4 - 1.0):
    return gamm1 * (q[4] - 0.5 * (q[1] * q[1] + q[2] * q[2] + q[3] * q[3]) / q[0])


def test_cp_field(case):
    mach = case.cfg.mach
    for mb in range(case.cfg.nblocks):
        q = case.get_state(mb)
        ref = (pressure(q) - 1.0 / 1.4) * (2.0 / mach ** 2)
        np.testing.assert_allclose(case.cp(mb), ref, rtol=1e-12, atol=1e-12)


def test_wall_probe_records_last_steps(case):
    case.wall_probe(4)
    case.step(7)
    t, p = case.wall_probe_read()
    assert p.shape[0] == 4 and t.shape == (4,)
    assert np.all(np.diff(t) > 0)
    assert abs(t[-1] - case.get_time()[5]) == 0.0
    # the last record is the wall pressure of the current state, mid-span line of each wall face
    cols = []
    for mb, ip in ((1, 1), (4, 0)):  # wall on top of block 1 and under block 4
        lxi, let, lze, _ = case.dims[mb]
        q = case.get_state(mb).reshape(5, lze + 1, let + 1, lxi + 1)
        cols.append(pressure(q[:, lze // 2, ip * let, :]))
    np.testing.assert_allclose(p[-1], np.concatenate(cols), rtol=1e-13, atol=0)
    case.wall_probe(0)


def test_restart_roundtrip_and_layout(case, tmp_path):
    nb = case.cfg.nblocks
    t0 = case.get_time()
    q0 = [case.get_state(mb).copy() for mb in range(nb)]
    for mb in range(nb):
        case.write_restart(mb, tmp_path / f"restart{mb:02d}.dat")
    # the reference's layout: 6 x 8-byte header slots, then qa(0:lmx,1:5) float64
    raw = np.fromfile(tmp_path / "restart01.dat", dtype=np.uint8)
    npts = case.npts(1)
    assert raw.size == 48 + 40 * npts
    assert raw[:4].view(np.int32)[0] == t0[0] and raw[8:12].view(np.int32)[0] == t0[1]
    np.testing.assert_array_equal(raw[16:48].view(np.float64), np.array(t0[2:]))
    np.testing.assert_array_equal(raw[48:].view(np.float64).reshape(5, -1), q0[1])
    # continue, come back, and the run repeats bit for bit
    case.step(3)
    q3 = [case.get_state(mb).copy() for mb in range(nb)]
    for mb in range(nb):
        case.read_restart(mb, tmp_path / f"restart{mb:02d}.dat")
    assert case.get_time() == t0
    for mb in range(nb):
        np.testing.assert_array_equal(case.get_state(mb), q0[mb])
    case.step(3)
    for mb in range(nb):
        np.testing.assert_array_equal(case.get_state(mb), q3[mb])


def read_plot3d(path, nvar, nhead):
    raw = np.fromfile(path, dtype=np.uint8)
    nb = raw[:4].view(np.int32)[0]
    dims = raw[4:4 + 12 * nb].view(np.int32).reshape(nb, 3)
    pos = 4 + 12 * nb
    out = []
    for b in range(nb):
        n = int(np.prod(dims[b]))
        head = raw[pos:pos + 4 * nhead].view(np.float32)
        pos += 4 * nhead
        data = raw[pos:pos + 4 * nvar * n].view(np.float32).reshape(nvar, n)
        pos += 4 * nvar * n
        out.append((head, data))
    assert pos == raw.size
    return dims, out


def test_plot3d_grid_and_solution(case, tmp_path):
    from tandemproject_gb300.grid import aerofoil_grid
    from tandemproject_gb300.solver import F_P
    nb = case.cfg.nblocks
    case.write_plot3d_grid(tmp_path / "grid.xyz")
    dims, blocks = read_plot3d(tmp_path / "grid.xyz", 3, 0)
    grid = aerofoil_grid(case.cfg)
    for mb in range(nb):
        lxi, let, lze, n = case.dims[mb]
        assert tuple(dims[mb]) == (lxi + 1, let + 1, lze + 1)
        np.testing.assert_array_equal(blocks[mb][1], grid[mb].reshape(3, -1).astype(np.float32))
    case.write_plot3d_solution(tmp_path / "sol.q")
    dims, blocks = read_plot3d(tmp_path / "sol.q", 5, 4)
    umf, aoa = case.frame()
    t = case.get_time()
    for mb in range(nb):
        head, data = blocks[mb]
        np.testing.assert_allclose(head, np.array([case.cfg.mach, aoa, case.cfg.reoo, t[5]], dtype=np.float32))
        q = case.get_state(mb)
        np.testing.assert_array_equal(data[0], q[0].astype(np.float32))
        for m in range(1, 4):
            np.testing.assert_array_equal(data[m], (q[m] / q[0] + umf[m - 1]).astype(np.float32))
        np.testing.assert_array_equal(data[4], case.get_field(mb, F_P)[0].astype(np.float32))


def test_whole_state_copies_match_the_block_copies(case):
    """ati_get/set_state_all: one [5][points_total] array, blocks in handle order."""
    n = case.points_total()
    assert n == sum(case.npts(mb) for mb in range(case.cfg.nblocks))
    q = case.get_state_all()
    assert q.shape == (5, n)
    off = 0
    for mb in range(case.cfg.nblocks):
        np.testing.assert_array_equal(q[:, off:off + case.npts(mb)], case.get_state(mb))
        off += case.npts(mb)
    q2 = q.copy()
    q2[0] *= 1.0 + 1e-9
    case.set_state_all(q2)
    np.testing.assert_array_equal(case.get_state(2), q2[:, sum(case.npts(mb) for mb in range(2)):][:, :case.npts(2)])
    case.set_state_all(q)
    np.testing.assert_array_equal(case.get_state_all(), q)
