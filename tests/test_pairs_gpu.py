"""Paired-line segmented derivative sweeps of the mixed path (k_sweep_pair).

A CTA solves two consecutive groups of 32 lines, lane l line l of each, with
each line's arithmetic written as in the one-group kernel (k_sweep_seg), so
the results must be bit-identical with the option on and off.  The cases cover
lines of one segment (one warp takes a 64-line tile) and of several (one warp
per segment, two 32-line tiles of a run whose odd length the host evens with a
padding tile), eta row tiles staged by TMA and per-thread copies, and a batch
of cases of different line lengths.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cases():
    from tandemproject_gb300.config import MIXED, small_case
    return [
        # aligned: TMA in eta and zeta; xi lines of 32 and 64 points (one and two segments)
        small_case(lxibk=(31, 63, 31), letbk=(15, 15), lzebk=(15,), precision=MIXED),
        # unaligned: per-thread copies; xi runs of 7 tiles (padded to 8) with two-segment lines
        small_case(precision=MIXED),
        # eta lines of 96 points (two segments) in TMA row tiles, rows of 32 lines (odd runs padded per row)
        # and of 64
        small_case(lxibk=(31, 63, 31), letbk=(95, 95), lzebk=(15,), precision=MIXED),
        # xi lines of 64 and 200 points (two and five segments), eta lines of 100 (three segments) in TMA row
        # tiles of 7 tiles a 200-point row, zeta lines of 60 points (two segments, runs of 625 tiles padded)
        small_case(lxibk=(63, 199, 63), letbk=(99, 99), lzebk=(59,), precision=MIXED),
    ]


@pytest.mark.parametrize("which", range(4))
def test_paired_lines_bit_identical(ati_lib, which):
    from tandemproject_gb300.solver import setup_case
    cfg = _cases()[which]
    a = setup_case(cfg)
    b = setup_case(cfg)
    assert a.set_options(paired_lines=True)["paired_lines"]
    assert not b.set_options(paired_lines=False)["paired_lines"]
    a.step(8)
    b.step(8)
    for mb in range(cfg.nblocks):
        assert np.array_equal(a.get_state(mb), b.get_state(mb)), mb
    # with TMA off as well (eta row tiles stay; the tiles come in by per-thread copies)
    a.set_options(tma=False, paired_lines=True)
    b.set_options(tma=False, paired_lines=False)
    a.step(3)
    b.step(3)
    for mb in range(cfg.nblocks):
        assert np.array_equal(a.get_state(mb), b.get_state(mb)), mb
    a.close()
    b.close()


def test_paired_lines_in_a_batch(ati_lib):
    from tandemproject_gb300.solver import setup_batch
    cfgs = _cases()
    a = setup_batch(cfgs)
    b = setup_batch(cfgs)
    a.set_options(paired_lines=True)
    b.set_options(paired_lines=False)
    a.step(5)
    b.step(5)
    for blk in range(sum(c.nblocks for c in cfgs)):
        assert np.array_equal(a.get_state(blk), b.get_state(blk)), blk
    a.close()
    b.close()
