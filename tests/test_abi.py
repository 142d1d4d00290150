"""The C-ABI library loads and exports every entry point include/ati.h
declares (no compute calls: these tests run without a GPU)."""
import ctypes
import os
import re

from conftest import ROOT


def declared(header):
    src = open(header).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char \*|void)\s*\*?\s*(ati_\w+|orc_\w+)\s*\(", src, re.M)))


def test_header_parses():
    names = declared(os.path.join(ROOT, "include", "ati.h"))
    assert "ati_create" in names and "ati_step" in names and "ati_deriv" in names


def test_library_exports_every_declared_symbol(ati_lib):
    lib = ctypes.CDLL(ati_lib)
    missing = [n for n in declared(os.path.join(ROOT, "include", "ati.h")) if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header(ati_lib):
    from tandemproject_gb300 import solver
    names = set(declared(os.path.join(ROOT, "include", "ati.h")))
    assert names <= set(solver.SIGNATURES), names - set(solver.SIGNATURES)
    lib = solver.load_library(ati_lib)
    assert lib.ati_abi_version() == 2


def test_oracle_exports_every_declared_symbol(oracle_lib):
    lib = ctypes.CDLL(oracle_lib)
    missing = [n for n in declared(os.path.join(ROOT, "oracle", "ati_oracle.h")) if not hasattr(lib, n)]
    assert not missing, missing


def test_config_struct_matches_header():
    """The ctypes mirror of ati_config_t has the C layout: 39 int32 (156 B, padded
    to 160) then 31 doubles; the turbulence fields took reserved slots, so the
    size is unchanged."""
    import ctypes as ct
    from tandemproject_gb300.config import AtiConfig
    assert ct.sizeof(AtiConfig) == 160 + 31 * 8
    assert AtiConfig.turb_modes.offset == 32 * 4 and AtiConfig.reoo.offset == 160
    assert AtiConfig.turb_intensity.offset == 160 + 23 * 8


def test_create_fails_loudly_without_gpu(ati_lib):
    """No CPU fallback: on a machine without a CUDA device ati_create refuses."""
    import pytest
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        pytest.skip("a GPU is present")
    from tandemproject_gb300.config import small_case
    from tandemproject_gb300.solver import AtiError, Case
    with pytest.raises(AtiError) as ei:
        Case(small_case())
    assert ei.value.code == 3
