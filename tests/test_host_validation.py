"""Argument checks that run on the host before any device work (no GPU
needed), each returning ATI_EINVAL with a message naming what is wrong:
- ati_create / ati_create_batch: the aerofoil H-grid topology, the RK stage
  count, the precision, a batch whose cases differ in their numerics, a batch
  of more blocks than a handle holds;
- ati_deriv_lines_noalloc: null arrays, a negative line count, lines shorter
  than the 7-point closures or longer than ATI_NOALLOC_MAX_LEN, more points
  than ATI_NOALLOC_MAX_POINTS; an empty call returns ATI_OK untouched.
No call here reaches a pointer: every case is refused (or empty) first."""
import ctypes

import pytest

ATI_EINVAL = 1


def _create(lib, cfgs):
    from tandemproject_gb300.config import AtiConfig
    arr = (AtiConfig * len(cfgs))(*cfgs)
    h = ctypes.c_void_p()
    if len(cfgs) == 1:
        rc = lib.ati_create(ctypes.byref(arr[0]), ctypes.byref(h))
    else:
        rc = lib.ati_create_batch(arr, len(cfgs), ctypes.byref(h))
    msg = lib.ati_last_error(None)
    return rc, (msg or b"").decode(), h.value


@pytest.fixture(scope="module")
def lib(ati_lib):
    from tandemproject_gb300.solver import load_library
    return load_library(ati_lib)


def _cfg(**kw):
    from tandemproject_gb300.config import small_case
    c = small_case().to_c()
    for k, v in kw.items():
        setattr(c, k, v)
    return c


@pytest.mark.parametrize("field,value,words", [
    ("bkx", 2, "bkx=3"),
    ("bkz", 2, "bkz=1"),
    ("nkrk", 0, "nkrk"),
    ("nkrk", 9, "nkrk"),
    ("precision", 7, "precision"),
])
def test_bad_case_rejected(lib, field, value, words):
    rc, msg, h = _create(lib, [_cfg(**{field: value})])
    assert rc == ATI_EINVAL and words in msg and not h


def test_batch_of_differing_numerics_rejected(lib):
    rc, msg, h = _create(lib, [_cfg(), _cfg(nviscous=0)])
    assert rc == ATI_EINVAL and "case 1 differs" in msg and not h


def test_batch_past_the_block_limit_rejected(lib):
    from tandemproject_gb300.config import AtiConfig
    n = 171  # six blocks a case: 1,026 blocks, past the 1,024 a handle holds
    arr = (AtiConfig * n)(*([_cfg()] * n))
    h = ctypes.c_void_p()
    rc = lib.ati_create_batch(arr, n, ctypes.byref(h))
    assert rc == ATI_EINVAL and b"too many cases" in lib.ati_last_error(None) and not h.value


def test_empty_batch_rejected(lib):
    from tandemproject_gb300.config import AtiConfig
    h = ctypes.c_void_p()
    rc = lib.ati_create_batch((AtiConfig * 1)(), 0, ctypes.byref(h))
    assert rc == ATI_EINVAL and not h.value


@pytest.mark.parametrize("args,words", [
    ((None, 16, 1, 10), b"null pointer"),
    ((16, None, 1, 10), b"null pointer"),
    ((16, 16, -1, 10), b"negative line count"),
    ((16, 16, 1, 6), b"line length"),
    ((16, 16, 1, 4097), b"ATI_NOALLOC_MAX_LEN"),
    ((16, 16, 200_001, 10), b"ATI_NOALLOC_MAX_POINTS"),
])
def test_noalloc_arguments_rejected(lib, args, words):
    src, dst, nlines, n = args
    rc = lib.ati_deriv_lines_noalloc(ctypes.c_void_p(src), ctypes.c_void_p(dst), nlines, n, None)
    assert rc == ATI_EINVAL and words in lib.ati_last_error(None)


def test_noalloc_empty_call(lib):
    assert lib.ati_deriv_lines_noalloc(ctypes.c_void_p(16), ctypes.c_void_p(16), 0, 10, None) == 0
