"""CUDA path vs the CPU oracle on the same seeded inputs, through the C ABI.

Tolerances (normwise relative error max|gpu-oracle|/max|oracle|):
  * set-up (metrics, Jacobian, normals, GCBC weights) and every granular
    deriv / filte / mpigo call run the no-contraction kernel build and must
    match the oracle bit for bit (tolerance 0); the bound of the reference
    contract is 1e-12 per call
  * fused steps (FMA contraction): relative L2 1e-10 per conserved variable
  * fused steps in ATI_FP64_STRICT: relative L2 1e-13 (only libm sin/pow differ)
Relative L2 is taken over all blocks; the three momentum components are
normalised by the L2 norm of the momentum vector (rho u, rho v, rho w), since
on a spanwise-extruded grid rho w stays orders of magnitude below rho u.
"""
import numpy as np
import pytest

from conftest import rel_err, rel_l2
from tandemproject_gb300.config import small_case
from tandemproject_gb300.grid import aerofoil_grid

pytestmark = pytest.mark.gpu

TOL_CALL = 1e-12
TOL_EXACT = 0.0
TOL_STEP = 1e-10
TOL_STRICT = 1e-13


def pair(cfg, grid=None):
    from oracle.oracle import OracleCase
    from tandemproject_gb300.solver import Case
    g = aerofoil_grid(cfg) if grid is None else grid
    gpu, orc = Case(cfg), OracleCase(cfg)
    for mb in range(cfg.nblocks):
        gpu.set_grid(mb, g[mb])
        orc.set_grid(mb, g[mb])
    gpu.init()
    orc.init()
    return gpu, orc


@pytest.fixture(scope="module")
def small(ati_lib, oracle_lib):
    cfg = small_case()
    return pair(cfg)


def test_metrics_and_jacobian(small):
    gpu, orc = small
    for mb in range(6):
        for fid in (5, 6, 7, 9):
            e = rel_err(gpu.get_field(mb, fid), orc.get_field(mb, fid))
            assert e <= TOL_EXACT, (mb, fid, e)


def test_face_normals_and_sponge(small):
    gpu, orc = small
    for mb in range(6):
        for nn in (1, 2, 3):
            assert rel_err(gpu.get_face(mb, 3, nn), orc.get_face(mb, 3, nn)) <= TOL_EXACT
        # sponge profiles use cos(): CUDA's and the C library's may differ in the last bit
        assert rel_err(gpu.get_field(mb, 11), orc.get_field(mb, 11)) < 1e-15


@pytest.mark.parametrize("nn", [1, 2, 3])
@pytest.mark.parametrize("nz", [1, 2, 3])
def test_deriv_each_direction(small, nn, nz):
    gpu, orc = small
    rng = np.random.default_rng(100 * nn + nz)
    for mb in range(6):
        r = rng.standard_normal((3, gpu.npts(mb)))
        gpu.set_field(mb, 3, r)
        orc.set_field(mb, 3, r)
    for c in (gpu, orc):
        c.mpigo(0, 0, 0)
        c.deriv(nn, nz, 2)
    for mb in range(6):
        assert rel_err(gpu.get_field(mb, 3), orc.get_field(mb, 3)) <= TOL_EXACT, mb
        fd, fo = gpu.get_face(mb, 0, nn), orc.get_face(mb, 0, nn)
        assert rel_err(fd[[1, 6]], fo[[1, 6]]) <= TOL_EXACT  # drva(:,m=2,0:1)
        if nn == 3:  # periodic closure received by mpigo
            assert rel_err(gpu.get_face(mb, 2, nn), orc.get_face(mb, 2, nn)) <= TOL_EXACT


@pytest.mark.parametrize("nn", [1, 2, 3])
def test_filte_each_direction(small, nn):
    gpu, orc = small
    rng = np.random.default_rng(7 + nn)
    for mb in range(6):
        r = rng.standard_normal((3, gpu.npts(mb)))
        gpu.set_field(mb, 3, r)
        orc.set_field(mb, 3, r)
    for c in (gpu, orc):
        c.mpigo(1, 1, 0)
        c.filte(nn, 1)
    for mb in range(6):
        assert rel_err(gpu.get_field(mb, 3), orc.get_field(mb, 3)) <= TOL_EXACT, mb


def test_mpigo_periodic_rebase(small):
    """n45 = 1 re-bases the periodic closure with the face value (metrics)."""
    gpu, orc = small
    rng = np.random.default_rng(3)
    for mb in range(6):
        r = rng.standard_normal((3, gpu.npts(mb)))
        gpu.set_field(mb, 3, r)
        orc.set_field(mb, 3, r)
    for c in (gpu, orc):
        c.mpigo(0, 1, 1)
    for mb in range(6):
        assert rel_err(gpu.get_face(mb, 2, 3), orc.get_face(mb, 2, 3)) <= TOL_EXACT


def test_deriv_of_constant_is_zero(small):
    gpu, _ = small
    for mb in range(6):
        gpu.set_field(mb, 3, np.full((3, gpu.npts(mb)), 2.5))
    gpu.mpigo(0, 1, 0)
    gpu.deriv(1, 1, 1)
    gpu.deriv(2, 1, 1)
    for mb in range(6):
        r = gpu.get_field(mb, 3)
        assert np.all(r[0] == 0.0) and np.all(r[1] == 0.0)


def state_errors(gpu, orc, nb=6):
    """Relative L2 per conserved variable over all blocks (momentum components
    against the momentum-vector norm)."""
    num = np.zeros(5)
    den = np.zeros(5)
    for mb in range(nb):
        q, qo = gpu.get_state(mb), orc.get_state(mb)
        num += np.sum((q - qo) ** 2, axis=1)
        den += np.sum(qo ** 2, axis=1)
    mom = den[1:4].sum()
    den[1:4] = mom
    return np.sqrt(num / np.maximum(den, 1e-300))


@pytest.fixture(scope="module")
def clean(ati_lib, oracle_lib):
    cfg = small_case(lxibk=(48, 120, 48), letbk=(39, 39), lzebk=(12,))
    return pair(cfg)


@pytest.mark.parametrize("strict", [False, True])
def test_one_stage_from_developed_state(ati_lib, oracle_lib, strict):
    """One filter + RK stage 1 from the same developed state (12 steps of the
    oracle copied into the GPU case): state, pressure, stresses and RHS.

    The RHS de is the sum of three flux derivatives that nearly cancel, so in
    the FMA build its normwise error is amplified (bound 1e-9) while the
    updated state stays at round-off; the strict build holds 1e-12 on all."""
    from tandemproject_gb300.config import FP64, FP64_STRICT
    cfg = small_case(lxibk=(48, 120, 48), letbk=(39, 39), lzebk=(12,), precision=FP64_STRICT if strict else FP64)
    gpu, orc = pair(cfg)
    assert orc.step(12) == 0
    for mb in range(6):
        gpu.set_field(mb, 0, orc.get_field(mb, 0))
        gpu.set_field(mb, 1, orc.get_field(mb, 1))
    gpu.set_time(orc.get_time())
    for c in (gpu, orc):
        c.filter_step()
        c.rk_stage(1)
    errs = {}
    for mb in range(6):
        for fid in (0, 2, 8, 10):
            errs[(mb, fid)] = rel_err(gpu.get_field(mb, fid), orc.get_field(mb, fid))
    print("one stage worst", "strict" if strict else "fast", max(errs.values()))
    for (mb, fid), e in errs.items():
        tol = 1e-9 if (fid == 2 and not strict) else 1e-12
        assert e < tol, (mb, fid, e)


def test_twenty_steps(clean):
    gpu, orc = clean
    gpu.step(19)
    assert orc.step(19) == 0
    tg, to = gpu.get_time(), orc.get_time()
    assert tg[0] == to[0] and tg[1] == to[1]
    assert abs(tg[2] - to[2]) <= 1e-12 * abs(to[2])
    e = state_errors(gpu, orc)
    print("19 steps rel L2", e)
    assert np.all(e < TOL_STEP), e
    fg, fo = gpu.forces(), orc.forces()
    assert np.allclose(fg, fo, rtol=1e-9, atol=1e-12), (fg, fo)


def test_strict_mode_steps(ati_lib, oracle_lib):
    """ATI_FP64_STRICT: no FMA contraction in the fused step either."""
    from tandemproject_gb300.config import FP64_STRICT
    cfg = small_case(lxibk=(48, 120, 48), letbk=(39, 39), lzebk=(12,), precision=FP64_STRICT)
    gpu, orc = pair(cfg)
    gpu.step(2)
    orc.step(2)
    # dt = 0 for the first two steps: no libm call differs, so the results are identical
    assert np.all(state_errors(gpu, orc) == 0.0)
    gpu.step(10)
    orc.step(10)
    e = state_errors(gpu, orc)
    print("strict 12 steps rel L2", e)
    assert np.all(e < TOL_STRICT), e


def test_naca0012_0p6m_hundred_steps(ati_lib, oracle_lib):
    """The reference contract: 1e-10 relative L2 per conserved variable after
    100 RK4 steps of the 0.6 M-point NACA 0012 case."""
    from tandemproject_gb300.config import PRESETS
    cfg = PRESETS["naca0012_0p6m"]
    gpu, orc = pair(cfg)
    gpu.step(100)
    assert orc.step(100) == 0
    e = state_errors(gpu, orc)
    print("naca0012_0p6m 100 steps rel L2", e)
    assert np.all(e < TOL_STEP), e


@pytest.mark.parametrize("precision", ["fp64", "strict"])
def test_les_branch_steps(ati_lib, oracle_lib, precision):
    """The Smagorinsky branch of the stresses (les = 1, src/Main3D.f90:656-678):
    19 steps against the oracle's restatement of the same branch.  The model
    constants are raised far above the deck's (0.16, 0.0066) so that the eddy
    viscosity changes the answer within these steps (by ~2e-7 on momentum; with
    the deck's constants by ~3e-14): the test is on the branch's arithmetic,
    not on the physics."""
    from tandemproject_gb300.config import FP64, FP64_STRICT
    prec = FP64_STRICT if precision == "strict" else FP64
    cfg = small_case(lxibk=(48, 120, 48), letbk=(39, 39), lzebk=(12,), les=1, precision=prec, smago1=400.0,
                     smago2=40.0)
    gpu, orc = pair(cfg)
    gpu.step(19)
    assert orc.step(19) == 0
    e = state_errors(gpu, orc)
    print("LES 19 steps rel L2", precision, e)
    assert np.all(e < (TOL_STRICT if precision == "strict" else TOL_STEP)), e
    # the branch changes the answer: the same case without it is measurably different
    cfg0 = cfg.replace(les=0)
    gpu0, _ = pair(cfg0)
    gpu0.step(19)
    diff = state_errors(gpu0, orc)
    print("LES on vs off after 19 steps", diff)
    assert np.any(diff > 1e-9)


def test_les_branch_mixed(ati_lib):
    """The mixed path's FP32 Smagorinsky branch tracks the FP64 one."""
    from tandemproject_gb300.config import MIXED
    from tandemproject_gb300.solver import setup_case
    cfg = small_case(lxibk=(48, 120, 48), letbk=(39, 39), lzebk=(12,), les=1, smago1=400.0, smago2=40.0)
    d, m = setup_case(cfg), setup_case(cfg.replace(precision=MIXED))
    d.step(19)
    m.step(19)
    e = state_errors(m, d)
    print("LES mixed vs fp64 19 steps", e)
    assert np.all(e < 1e-5), e


def test_newton_reciprocal_and_rsqrt_bounds(ati_lib):
    """The FP64 fast build's primitives take 1/rho, 1/(T + S) and 1/sqrt(T) from
    hardware approximations refined by two Newton-Raphson steps; over 2^24
    arguments they stay within 4 x 2^-53 of the IEEE division and square root."""
    import ctypes
    from tandemproject_gb300.solver import load_library
    L = load_library(ati_lib)
    worst = (ctypes.c_double * 2)(-1.0, -1.0)
    assert L.ati_check_recip(1 << 24, worst) == 0
    print("Newton reciprocal / rsqrt, worst relative difference", worst[0], worst[1])
    assert 0.0 <= worst[0] <= 4 * 2.0 ** -53
    assert 0.0 <= worst[1] <= 4 * 2.0 ** -53


@pytest.mark.parametrize("lxibk", [(24, 64, 24), (48, 120, 48)])
def test_fp64_stresses_at_the_point_bit_identical(ati_lib, lxibk):
    """The ATI_FP64 path's viscous fluxes with the stresses of k_visc taken at the
    point (ATI_OPT_STRESS_AT_POINT, on by default) round exactly as the stress
    planes written by k_visc and read by k_flux: states bit for bit after 12
    steps, and the stress output rebuilt on demand equals the planes."""
    from tandemproject_gb300.config import FP64
    from tandemproject_gb300.solver import setup_case
    cfg = small_case(lxibk=lxibk, letbk=(39, 39), lzebk=(12,), precision=FP64)
    a, b = setup_case(cfg), setup_case(cfg)
    assert a.set_options(stress_at_point=True)["stress_at_point"]
    assert not b.set_options(stress_at_point=False)["stress_at_point"]
    a.step(12)
    b.step(12)
    for mb in range(cfg.nblocks):
        assert np.array_equal(a.get_state(mb), b.get_state(mb)), mb
        assert np.array_equal(a.get_field(mb, 10), b.get_field(mb, 10)), mb
    assert np.array_equal(a.forces(), b.forces())
    a.close()
    b.close()
