"""ctypes binding of the CPU oracle (test infrastructure only).

Only tests/, the smoke check of __graft_entry__.py and the CPU-baseline leg of
bench.py import this module.  The product never does.
"""
import ctypes
import os

import numpy as np

from . import build as _build
from tandemproject_gb300.config import AtiTime, CaseConfig

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = ctypes.CDLL(path)
        vp, i32, dp = ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double)
        L.orc_create.argtypes = [vp, ctypes.POINTER(vp)]
        L.orc_destroy.argtypes = [vp]
        L.orc_destroy.restype = None
        for name, args in [("orc_set_grid", [vp, i32, dp]), ("orc_init", [vp]),
                           ("orc_set_field", [vp, i32, i32, dp]), ("orc_get_field", [vp, i32, i32, dp]),
                           ("orc_get_face", [vp, i32, i32, i32, dp]), ("orc_mpigo", [vp, i32, i32, i32]),
                           ("orc_deriv", [vp, i32, i32, i32]), ("orc_filte", [vp, i32, i32]),
                           ("orc_filter_step", [vp]), ("orc_rk_stage", [vp, i32]), ("orc_step", [vp, i32]),
                           ("orc_forces", [vp, dp]), ("orc_get_time", [vp, vp]), ("orc_set_time", [vp, vp]),
                           ("orc_scheme", [vp, i32, dp]), ("orc_factors", [vp, i32, i32, i32, dp, dp]),
                           ("orc_topology", [vp, i32, vp, vp]), ("orc_block_dims", [vp, i32, vp, vp])]:
            f = getattr(L, name)
            f.argtypes = args
            f.restype = ctypes.c_int
        L.orc_set_turbulence.argtypes = [vp, ctypes.c_void_p, i32]
        L.orc_set_turbulence.restype = ctypes.c_int
        L.orc_build_modes.argtypes = [vp, ctypes.c_void_p]
        L.orc_build_modes.restype = ctypes.c_int
        L.orc_set_threads.argtypes = [ctypes.c_int]
        L.orc_set_threads.restype = None
        L.orc_get_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


NCOMP = {0: 5, 1: 5, 2: 5, 3: 3, 4: 3, 5: 3, 6: 3, 7: 3, 8: 1, 9: 1, 10: 9, 11: 2}


class OracleCase:
    """One case on the CPU oracle, same call surface as the CUDA Case."""

    def __init__(self, cfg: CaseConfig):
        self.cfg = cfg
        self._c = cfg.to_c()
        h = ctypes.c_void_p()
        rc = lib().orc_create(ctypes.byref(self._c), ctypes.byref(h))
        if rc:
            raise RuntimeError(f"orc_create failed: {rc}")
        self.h = h
        self.dims = []
        for mb in range(cfg.nblocks):
            d = (ctypes.c_int32 * 3)()
            n = ctypes.c_int64()
            lib().orc_block_dims(self.h, mb, d, ctypes.byref(n))
            self.dims.append((d[0], d[1], d[2], n.value))

    def close(self):
        if self.h:
            lib().orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _chk(self, rc, what):
        if rc:
            raise RuntimeError(f"{what} failed with status {rc}")

    def npts(self, mb):
        return self.dims[mb][3]

    def set_grid(self, mb, xyz):
        a = np.ascontiguousarray(xyz, dtype=np.float64)
        self._chk(lib().orc_set_grid(self.h, mb, _dp(a)), "orc_set_grid")

    def init(self):
        self._chk(lib().orc_init(self.h), "orc_init")

    def get_field(self, mb, fid):
        out = np.empty(NCOMP[fid] * self.npts(mb))
        self._chk(lib().orc_get_field(self.h, mb, fid, _dp(out)), "orc_get_field")
        return out.reshape(NCOMP[fid], -1)

    def set_field(self, mb, fid, v):
        a = np.ascontiguousarray(v, dtype=np.float64).ravel()
        self._chk(lib().orc_set_field(self.h, mb, fid, _dp(a)), "orc_set_field")

    def get_state(self, mb):
        return self.get_field(mb, 0)

    def set_state(self, mb, q):
        self.set_field(mb, 0, q)

    def get_face(self, mb, which, nn):
        lxi, let, lze, _ = self.dims[mb]
        nbs = {1: (let + 1) * (lze + 1), 2: (lze + 1) * (lxi + 1), 3: (lxi + 1) * (let + 1)}[nn]
        nc = 10 if which in (0, 1) else 6
        out = np.empty(nc * nbs)
        self._chk(lib().orc_get_face(self.h, mb, which, nn, _dp(out)), "orc_get_face")
        return out.reshape(-1, nbs)

    def mpigo(self, nt, nrt, n45):
        self._chk(lib().orc_mpigo(self.h, nt, nrt, n45), "orc_mpigo")

    def deriv(self, nn, nz, m):
        self._chk(lib().orc_deriv(self.h, nn, nz, m), "orc_deriv")

    def filte(self, nn, nz):
        self._chk(lib().orc_filte(self.h, nn, nz), "orc_filte")

    def filter_step(self):
        self._chk(lib().orc_filter_step(self.h), "orc_filter_step")

    def rk_stage(self, nk):
        self._chk(lib().orc_rk_stage(self.h, nk), "orc_rk_stage")

    def step(self, n=1):
        return lib().orc_step(self.h, n)

    def forces(self):
        out = np.zeros(2)
        self._chk(lib().orc_forces(self.h, _dp(out)), "orc_forces")
        return out

    def set_turbulence(self, modes):
        """Inflow turbulence from a (nmodes, 8) float32 mode table (Case.turbulence_modes()), after init."""
        m = np.ascontiguousarray(modes, dtype=np.float32)
        self._modes = m
        self._chk(lib().orc_set_turbulence(self.h, m.ctypes.data_as(ctypes.c_void_p), int(m.shape[0])),
                  "orc_set_turbulence")

    def get_time(self):
        t = AtiTime()
        lib().orc_get_time(self.h, ctypes.byref(t))
        return t.as_tuple()

    def set_time(self, tup):
        t = AtiTime(*tup)
        lib().orc_set_time(self.h, ctypes.byref(t))

    def scheme(self, which, n):
        out = np.zeros(n)
        self._chk(lib().orc_scheme(self.h, which, _dp(out)), "orc_scheme")
        return out

    def factors(self, mb, nn, filt):
        lxi, let, lze, _ = self.dims[mb]
        ln = {1: lxi, 2: let, 3: lze}[nn] + 1
        u = np.zeros(3 * ln)
        l = np.zeros(2 * ln)
        self._chk(lib().orc_factors(self.h, mb, nn, filt, _dp(u), _dp(l)), "orc_factors")
        return u.reshape(3, ln), l.reshape(2, ln)

    def topology(self, mb):
        nbc = (ctypes.c_int32 * 6)()
        ncd = (ctypes.c_int32 * 6)()
        lib().orc_topology(self.h, mb, nbc, ncd)
        return list(nbc), list(ncd)


def build_modes(cfg):
    """(nmodes, 8) float32 inflow-turbulence mode table of cfg (empty without turbulence)."""
    c = cfg.to_c()
    n = lib().orc_build_modes(ctypes.byref(c), None)
    out = np.zeros((n, 8), dtype=np.float32)
    if n:
        lib().orc_build_modes(ctypes.byref(c), out.ctypes.data_as(ctypes.c_void_p))
    return out


def set_threads(n):
    lib().orc_set_threads(int(n))


def get_threads():
    return lib().orc_get_threads()
