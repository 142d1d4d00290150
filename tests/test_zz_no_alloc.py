"""The allocation-free derivative entry point (ati_deriv_lines_noalloc).

Some callers of this library cannot allocate GPU memory when they call in: a
host code that hands all device memory to its own pool at start-up, or a time
loop that must not allocate once it runs (an allocation can stall the device
or fail late).  This entry point serves them: its scratch is one fixed static
device array and the caller passes its own input and output arrays.

The test calls it through the C ABI four times in a row, on lines of two
lengths (the last call repeats the previous length, so it reuses the LU
factors that call left in the scratch array), and checks every result against
the handle-based ati_deriv along xi, which runs the same arithmetic: the
tolerance is the per-call parity bound 1e-12 (the two agree bit for bit).  It
also checks that calls after the first leave the device's free memory
unchanged.  This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

TOL = 1e-12


def test_noalloc_matches_deriv_consecutive_calls(ati_lib):
    import torch

    from tandemproject_gb300.config import small_case
    from tandemproject_gb300.grid import aerofoil_grid
    from tandemproject_gb300.solver import Case, load_library

    L = load_library(ati_lib)
    cfg = small_case()
    case = Case(cfg)
    g = aerofoil_grid(cfg)
    for mb in range(cfg.nblocks):
        case.set_grid(mb, g[mb])
    case.init()
    rng = np.random.default_rng(2024)
    inputs = []
    for mb in range(cfg.nblocks):
        r = rng.standard_normal((3, case.npts(mb)))
        case.set_field(mb, 3, r)
        inputs.append(r[0].copy())
    case.deriv(1, 1, 1)  # the handle-based entry point: d/dxi of rr(:,1) into rr(:,1)
    expected = [case.get_field(mb, 3)[0] for mb in range(cfg.nblocks)]
    stream = torch.cuda.current_stream()
    # every device array of the test is made before the first call, so free memory can only change through the calls
    order = (0, 1, 0, 0)  # xi lengths 25, 65, 25, 25
    bufs = {}
    for mb in set(order):
        din = torch.from_numpy(inputs[mb]).cuda()
        bufs[mb] = (din, torch.empty_like(din))
    torch.cuda.synchronize()
    free_after_first = None
    for n, mb in enumerate(order):
        lxi, let, lze, npts = case.dims[mb]
        nlines, ln = (let + 1) * (lze + 1), lxi + 1
        din, dout = bufs[mb]
        dout.fill_(float("nan"))
        torch.cuda.synchronize()
        rc = L.ati_deriv_lines_noalloc(ctypes.c_void_p(din.data_ptr()), ctypes.c_void_p(dout.data_ptr()),
                                       nlines, ln, ctypes.c_void_p(stream.cuda_stream))
        assert rc == 0, L.ati_last_error(None)
        torch.cuda.synchronize()
        got = dout.cpu().numpy()
        e = rel_err(got, expected[mb])
        assert e <= TOL, (n, mb, e)
        free = torch.cuda.mem_get_info()[0]
        if n == 0:
            free_after_first = free
        else:
            assert free == free_after_first, (n, free, free_after_first)
    case.close()


def test_noalloc_rejects_oversize(ati_lib):
    from tandemproject_gb300.solver import load_library
    L = load_library(ati_lib)
    # rejected on the host before any launch: too many points, and a too-long line
    rc = L.ati_deriv_lines_noalloc(ctypes.c_void_p(16), ctypes.c_void_p(16), 2_000_001, 10, None)
    assert rc == 1 and b"ATI_NOALLOC_MAX_POINTS" in L.ati_last_error(None)
    rc = L.ati_deriv_lines_noalloc(ctypes.c_void_p(16), ctypes.c_void_p(16), 1, 5000, None)
    assert rc == 1 and b"ATI_NOALLOC_MAX_LEN" in L.ati_last_error(None)
