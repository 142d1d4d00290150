"""Mixed precision (ATI_MIXED): line solves, filters and fluxes in FP32, FP64
metrics, Jacobian and RK state.  Errors are measured against the FP64 path,
which itself matches the CPU restatement to ~1e-14 after 100 steps."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def state_rel_l2(a, b, nb=6):
    num = np.zeros(5)
    den = np.zeros(5)
    for mb in range(nb):
        qa, qb = a.get_state(mb), b.get_state(mb)
        num += np.sum((qa - qb) ** 2, axis=1)
        den += np.sum(qb ** 2, axis=1)
    den[1:4] = den[1:4].sum()
    return np.sqrt(num / den)


def make(cfg):
    from tandemproject_gb300.solver import setup_case
    return setup_case(cfg)


def test_mixed_tracks_fp64(ati_lib):
    from tandemproject_gb300.config import MIXED, small_case
    cfg = small_case(lxibk=(48, 120, 48), letbk=(39, 39), lzebk=(12,))
    d = make(cfg)
    m = make(cfg.replace(precision=MIXED))
    d.step(2)
    m.step(2)
    e2 = state_rel_l2(m, d)
    d.step(98)
    m.step(98)
    e100 = state_rel_l2(m, d)
    print("mixed vs fp64 rel L2 after 2 steps", e2, "after 100 steps", e100)
    assert np.all(e2 < 1e-6)
    assert np.all(e100 < 1e-5)
    td, tm = d.get_time(), m.get_time()
    assert td[0] == tm[0] and abs(td[2] - tm[2]) < 1e-5 * td[2]
    fd, fm = d.forces(), m.forces()
    print("forces fp64", fd, "mixed", fm)
    assert np.allclose(fd, fm, rtol=1e-3, atol=1e-6)


def test_mixed_filter_step_matches_fp64_closely(ati_lib):
    """The FP32 filter adds an FP32 correction to the FP64 state."""
    from tandemproject_gb300.config import MIXED, small_case
    cfg = small_case(lxibk=(48, 120, 48), letbk=(39, 39), lzebk=(12,))
    d = make(cfg)
    m = make(cfg.replace(precision=MIXED))
    rng = np.random.default_rng(5)
    for mb in range(6):
        q = d.get_state(mb)
        # the initial state is at rest: give it momentum (a mean drift plus noise)
        q = q * (1.0 + 1e-3 * rng.standard_normal(q.shape))
        q[1] = q[0] * (0.2 + 1e-3 * rng.standard_normal(q.shape[1]))
        q[2] = q[0] * 1e-3 * rng.standard_normal(q.shape[1])
        q[3] = q[0] * 1e-3 * rng.standard_normal(q.shape[1])
        d.set_state(mb, q)
        m.set_state(mb, q)
    d.filter_step()
    m.filter_step()
    e = state_rel_l2(m, d)
    assert np.all(e < 1e-7), e
