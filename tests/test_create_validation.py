"""ati_create / ati_create_batch reject a bad configuration before they look
for a device, with ATI_EINVAL and a message naming the field (host logic,
no GPU needed): the aerofoil H-grid topology, the RK stage count, the
precision, a batch whose cases differ in their numerics, and a batch of
more blocks than a handle holds."""
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
