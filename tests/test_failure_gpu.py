"""Failure detection without a GPU fault.

The reference's only failure check is the dt = 0 "Overflow." stop
(src/Main3D.f90:552,1086-1090).  Here every case of a handle carries a device
flag for a non-finite or non-positive density or pressure, read by the host
after the step; the failure is made on the host (a NaN written into one case's
state), never by faulting the GPU.  Host waits can be bounded
(ati_set_wait_timeout): a wait that runs out returns ATI_ETIMEDOUT with the
work still in flight, and a later wait completes it.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ATI_ENONFINITE, ATI_ETIMEDOUT = 4, 5


def _cases():
    from tandemproject_gb300.config import small_case
    return [small_case(), small_case(lxibk=(32, 64, 32), letbk=(16, 20)), small_case(lzebk=(16,), mach=0.3)]


def test_nan_in_one_case_of_a_batch_leaves_the_others_untouched(ati_lib):
    from tandemproject_gb300.solver import AtiError, setup_batch, setup_case
    cfgs = _cases()
    b = setup_batch(cfgs)
    blk = b.block(1, 2)
    q = b.get_state(blk)
    q[0, q.shape[1] // 2] = np.nan
    b.set_state(blk, q)
    with pytest.raises(AtiError) as ei:
        b.step(6)
    assert ei.value.code == ATI_ENONFINITE and "case 1" in str(ei.value)
    b.case_check(0)
    b.case_check(2)
    with pytest.raises(AtiError) as ei:
        b.case_check(1)
    assert ei.value.code == ATI_ENONFINITE
    # the failed case keeps its own non-finite state; every other case is bit for bit its run alone
    assert not np.all(np.isfinite(np.concatenate([s.ravel() for s in b.case_state(1)])))
    for cs in (0, 2):
        solo = setup_case(cfgs[cs])
        solo.step(6)
        for mb in range(cfgs[cs].nblocks):
            assert np.array_equal(b.get_state(b.block(cs, mb)), solo.get_state(mb)), (cs, mb)
        assert b.case_time(cs) == solo.get_time()
        solo.close()
    # the batch goes on stepping; the healthy cases stay finite, the failed one stays flagged
    with pytest.raises(AtiError):
        b.step(2)
    b.case_check(0)
    b.case_check(2)
    b.close()


def test_bounded_wait_times_out_then_completes(ati_lib):
    from tandemproject_gb300.config import PRESETS
    from tandemproject_gb300.solver import AtiError, setup_case
    c = setup_case(PRESETS["naca0012_0p6m"])
    c.step(1)
    n0 = c.get_time()[0]
    c.set_wait_timeout(1e-6)
    c.step_async(30)
    with pytest.raises(AtiError) as ei:
        c.synchronize()
    assert ei.value.code == ATI_ETIMEDOUT
    with pytest.raises(AtiError) as ei:
        c.check()
    assert ei.value.code == ATI_ETIMEDOUT
    # ati_step issues its steps before the bounded wait: they are in flight when it times out
    with pytest.raises(AtiError) as ei:
        c.step(5)
    assert ei.value.code == ATI_ETIMEDOUT
    c.set_wait_timeout(0)
    c.check()
    c.synchronize()
    assert c.get_time()[0] == n0 + 35
    q = c.get_state(1)
    assert np.all(np.isfinite(q))
    # a generous limit does not time out
    c.set_wait_timeout(60.0)
    c.step(2)
    c.close()


def test_wait_timeout_rejects_bad_values(ati_lib):
    from tandemproject_gb300.config import small_case
    from tandemproject_gb300.solver import AtiError, Case
    c = Case(small_case())
    for v in (-1.0, float("nan")):
        with pytest.raises(AtiError):
            c.set_wait_timeout(v)
    c.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_fused_face_chains_bit_identical(ati_lib, precision):
    """The fused face chains (two cooperative launches a stage) give the per-face
    kernels' results bit for bit, on a batch of uneven cases."""
    from tandemproject_gb300.config import FP64, MIXED
    from tandemproject_gb300.solver import setup_batch
    prec = MIXED if precision == "mixed" else FP64
    cfgs = [c.replace(precision=prec) for c in _cases()]
    a = setup_batch(cfgs)
    b = setup_batch(cfgs)
    assert a.set_options(fused_faces=True)["fused_faces"]
    assert not b.set_options(fused_faces=False)["fused_faces"]
    a.step(9)
    b.step(9)
    for blk in range(sum(c.nblocks for c in cfgs)):
        assert np.array_equal(a.get_state(blk), b.get_state(blk)), blk
    a.close()
    b.close()


def test_device_barrier_wait_times_out(ati_lib):
    """A grid barrier of the fused face chains gives up after the handle's spin
    limit: with a limit of one poll the waiting CTAs stop, every case is marked
    and the step returns ATI_ETIMEDOUT; the handle stays usable (re-initialised,
    it steps normally)."""
    from tandemproject_gb300.config import small_case
    from tandemproject_gb300.solver import AtiError, setup_case
    c = setup_case(small_case())
    assert c.set_options(fused_faces=True)["fused_faces"]
    c.step(2)
    c.set_spin_limit(1)
    with pytest.raises(AtiError) as ei:
        c.step(4)
    assert ei.value.code == ATI_ETIMEDOUT
    with pytest.raises(AtiError) as ei:
        c.check()
    assert ei.value.code == ATI_ETIMEDOUT
    c.set_spin_limit(0)
    c.init()
    c.step(3)
    c.check()
    assert np.all(np.isfinite(c.get_state(0)))
    c.close()
