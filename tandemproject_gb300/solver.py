"""Host-side mirror of the reference's call surface over the CUDA library.

``Case`` owns one ``ati_handle_t`` (include/ati.h).  Its methods keep the
reference's names and selector arguments:

    mpigo(nt, nrt, n45)      src/Subroutines3D.f90:16-80
    deriv(nn, nz, m)         src/Subroutines3D.f90:84-141
    filte(nn, nz)            src/Subroutines3D.f90:145-206
    filter_step()            src/Main3D.f90:555-561
    rk_stage(nk)             src/Main3D.f90:567-958
    step(nsteps)             src/Main3D.f90:552-965
    forces()                 clpost, src/rpt.f90:1017-1056

There is no CPU fallback: if libati.so cannot be loaded, or no CUDA device is
present, construction raises.
"""
import ctypes
import os

import numpy as np

from .config import AtiTime, CaseConfig

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libati.so")

ATI_OK, ATI_EINVAL, ATI_ENOMEM, ATI_ECUDA, ATI_ENONFINITE, ATI_ETIMEDOUT, ATI_ESTATE = range(7)
F_QA, F_QO, F_DE, F_RR, F_SS, F_XIM, F_ETM, F_ZEM, F_P, F_YACO, F_STRESS, F_SPONGE, F_CP = range(13)
FACE_DRVA, FACE_DRVB, FACE_RECV, FACE_CM = range(4)
OPT_TMA, OPT_FUSED_FACES, OPT_TMA_ETA, OPT_TMA_ZETA, OPT_PAIRED_LINES, OPT_STRESS_AT_POINT = 1, 2, 4, 8, 16, 32
OPT_DENSE_ZETA = 64
TILE_PLAN = 11  # ATI_TILE_PLAN
NCOMP = {F_QA: 5, F_QO: 5, F_DE: 5, F_RR: 3, F_SS: 3, F_XIM: 3, F_ETM: 3, F_ZEM: 3, F_P: 1, F_YACO: 1,
         F_STRESS: 9, F_SPONGE: 2, F_CP: 1}

# every entry point declared in include/ati.h, with its ctypes signature
_vp, _i32, _dp = ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double)
SIGNATURES = {
    "ati_abi_version": ([], ctypes.c_int),
    "ati_create": ([_vp, ctypes.POINTER(_vp)], ctypes.c_int),
    "ati_destroy": ([_vp], ctypes.c_int),
    "ati_last_error": ([_vp], ctypes.c_char_p),
    "ati_synchronize": ([_vp], ctypes.c_int),
    "ati_set_grid": ([_vp, _i32, _dp], ctypes.c_int),
    "ati_init": ([_vp], ctypes.c_int),
    "ati_set_state": ([_vp, _i32, _dp], ctypes.c_int),
    "ati_get_state": ([_vp, _i32, _dp], ctypes.c_int),
    "ati_set_state_all": ([_vp, _dp], ctypes.c_int),
    "ati_get_state_all": ([_vp, _dp], ctypes.c_int),
    "ati_points_total": ([_vp, _vp], ctypes.c_int),
    "ati_set_field": ([_vp, _i32, _i32, _dp], ctypes.c_int),
    "ati_get_field": ([_vp, _i32, _i32, _dp], ctypes.c_int),
    "ati_get_face": ([_vp, _i32, _i32, _i32, _dp], ctypes.c_int),
    "ati_get_time": ([_vp, _vp], ctypes.c_int),
    "ati_set_time": ([_vp, _vp], ctypes.c_int),
    "ati_block_dims": ([_vp, _i32, _vp, _vp], ctypes.c_int),
    "ati_mpigo": ([_vp, _i32, _i32, _i32], ctypes.c_int),
    "ati_deriv": ([_vp, _i32, _i32, _i32], ctypes.c_int),
    "ati_filte": ([_vp, _i32, _i32], ctypes.c_int),
    "ati_filter_step": ([_vp], ctypes.c_int),
    "ati_rk_stage": ([_vp, _i32], ctypes.c_int),
    "ati_step": ([_vp, _i32], ctypes.c_int),
    "ati_forces": ([_vp, _dp], ctypes.c_int),
    "ati_profile_enable": ([_vp, _i32], ctypes.c_int),
    "ati_profile_read": ([_vp, _i32, _dp, _vp], ctypes.c_int),
    "ati_launch_count": ([_vp, _vp], ctypes.c_int),
    "ati_stream": ([_vp], ctypes.c_void_p),
    "ati_probe_fma_tflops": ([_i32, _dp], ctypes.c_int),
    "ati_deriv_lines_noalloc": ([_vp, _vp, ctypes.c_int64, ctypes.c_int32, _vp], ctypes.c_int),
    "ati_get_config": ([_vp, _vp], ctypes.c_int),
    "ati_get_frame": ([_vp, _dp, _dp], ctypes.c_int),
    "ati_wall_probe_enable": ([_vp, _i32], ctypes.c_int),
    "ati_wall_probe_read": ([_vp, _dp, _dp, _vp, _vp], ctypes.c_int),
    "ati_write_restart": ([_vp, _i32, ctypes.c_char_p], ctypes.c_int),
    "ati_read_restart": ([_vp, _i32, ctypes.c_char_p], ctypes.c_int),
    "ati_write_plot3d_grid": ([_vp, ctypes.c_char_p], ctypes.c_int),
    "ati_write_plot3d_solution": ([_vp, ctypes.c_char_p], ctypes.c_int),
    "ati_create_batch": ([_vp, _i32, ctypes.POINTER(_vp)], ctypes.c_int),
    "ati_step_async": ([_vp, _i32], ctypes.c_int),
    "ati_jacobian_sign": ([_vp, _vp], ctypes.c_int),
    "ati_tiles": ([_vp, _vp], ctypes.c_int),
    "ati_set_tuning": ([_vp, _i32], ctypes.c_int),
    "ati_get_tile_plan": ([_vp, _vp], ctypes.c_int),
    "ati_set_tile_plan": ([_vp, _vp], ctypes.c_int),
    "ati_set_tiles": ([_vp, _vp], ctypes.c_int),
    "ati_set_options": ([_vp, _i32, _vp], ctypes.c_int),
    "ati_set_spin_limit": ([_vp, ctypes.c_int64], ctypes.c_int),
    "ati_check_conversions": ([ctypes.c_int64, _vp], ctypes.c_int),
    "ati_check_recip": ([ctypes.c_int64, _dp], ctypes.c_int),
    "ati_dense_zeta_operator": ([_vp, _i32, _dp, _vp], ctypes.c_int),
    "ati_turbulence_modes": ([_vp, _i32, _vp, _vp], ctypes.c_int),
    "ati_turbulence_sample": ([_vp, _i32, ctypes.c_double, ctypes.c_int64, _dp, _dp], ctypes.c_int),
    "ati_query": ([_vp, _vp], ctypes.c_int),
    "ati_check": ([_vp], ctypes.c_int),
    "ati_case_check": ([_vp, _i32], ctypes.c_int),
    "ati_set_wait_timeout": ([_vp, ctypes.c_double], ctypes.c_int),
    "ati_case_count": ([_vp, _vp], ctypes.c_int),
    "ati_case_blocks": ([_vp, _i32, _vp, _vp], ctypes.c_int),
    "ati_case_time": ([_vp, _i32, _vp], ctypes.c_int),
    "ati_case_set_time": ([_vp, _i32, _vp], ctypes.c_int),
    "ati_case_config": ([_vp, _i32, _vp], ctypes.c_int),
    "ati_case_forces": ([_vp, _i32, _dp], ctypes.c_int),
    "ati_case_frame": ([_vp, _i32, _dp, _dp], ctypes.c_int),
}

KERNEL_CLASSES = ["deriv_xi", "deriv_eta", "deriv_zeta", "filter_xi", "filter_eta", "filter_zeta", "mpigo",
                  "prim", "cfl", "visc", "flux", "div", "rk", "gcbc", "wall_junction", "average", "scalar"]

_lib = None


def load_library(path=LIB_PATH):
    """Load libati.so and bind every entry point; raise if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"libati.so not built at {path}: run tandemproject_gb300.build.build() "
                           "(there is no CPU fallback)")
    L = ctypes.CDLL(path)
    for name, (args, res) in SIGNATURES.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _lib = L
    return L


def _dp_of(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class AtiError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"status {code}: {msg}")
        self.code = code


class Case:
    """One aerofoil case resident on the GPU (all blocks in one handle)."""

    def __init__(self, cfg: CaseConfig, lib_path=LIB_PATH):
        self.L = load_library(lib_path)
        self.cfg = cfg
        self._c = cfg.to_c()
        h = ctypes.c_void_p()
        rc = self.L.ati_create(ctypes.byref(self._c), ctypes.byref(h))
        if rc:
            raise AtiError(rc, self.L.ati_last_error(None).decode())
        self.h = h
        self._dims(cfg.nblocks)

    def _dims(self, nblocks):
        self.dims = []
        for mb in range(nblocks):
            d = (ctypes.c_int32 * 3)()
            n = ctypes.c_int64()
            self._chk(self.L.ati_block_dims(self.h, mb, d, ctypes.byref(n)))
            self.dims.append((d[0], d[1], d[2], n.value))

    # -- lifetime
    def close(self):
        if getattr(self, "h", None):
            self.L.ati_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _chk(self, rc):
        if rc:
            raise AtiError(rc, self.L.ati_last_error(self.h).decode())
        return rc

    def npts(self, mb):
        return self.dims[mb][3]

    # -- set-up
    def set_grid(self, mb, xyz):
        a = np.ascontiguousarray(xyz, dtype=np.float64)
        assert a.size == 3 * self.npts(mb)
        self._chk(self.L.ati_set_grid(self.h, mb, _dp_of(a)))

    def init(self):
        self._chk(self.L.ati_init(self.h))

    # -- copies
    def get_field(self, mb, fid):
        out = np.empty(NCOMP[fid] * self.npts(mb))
        self._chk(self.L.ati_get_field(self.h, mb, fid, _dp_of(out)))
        return out.reshape(NCOMP[fid], -1)

    def set_field(self, mb, fid, v):
        a = np.ascontiguousarray(v, dtype=np.float64).ravel()
        assert a.size == NCOMP[fid] * self.npts(mb)
        self._chk(self.L.ati_set_field(self.h, mb, fid, _dp_of(a)))

    def get_state(self, mb, out=None):
        if out is None:
            out = np.empty(5 * self.npts(mb))
        self._chk(self.L.ati_get_state(self.h, mb, _dp_of(out)))
        return out.reshape(5, -1)

    def set_state(self, mb, q):
        a = np.ascontiguousarray(q, dtype=np.float64)
        self._chk(self.L.ati_set_state(self.h, mb, _dp_of(a)))

    def points_total(self):
        n = ctypes.c_int64()
        self._chk(self.L.ati_points_total(self.h, ctypes.byref(n)))
        return n.value

    def get_state_all(self, out=None):
        """The state of every block, [5][points_total] with blocks in handle order, in one copy."""
        if out is None:
            out = np.empty(5 * self.points_total())
        assert out.dtype == np.float64 and out.flags.c_contiguous and out.size == 5 * self.points_total()
        self._chk(self.L.ati_get_state_all(self.h, _dp_of(out)))
        return out.reshape(5, -1)

    def set_state_all(self, q):
        a = np.ascontiguousarray(q, dtype=np.float64)
        assert a.size == 5 * self.points_total()
        self._chk(self.L.ati_set_state_all(self.h, _dp_of(a)))

    def get_face(self, mb, which, nn):
        lxi, let, lze, _ = self.dims[mb]
        nbs = {1: (let + 1) * (lze + 1), 2: (lze + 1) * (lxi + 1), 3: (lxi + 1) * (let + 1)}[nn]
        nc = 10 if which in (FACE_DRVA, FACE_DRVB) else 6
        out = np.empty(nc * nbs)
        self._chk(self.L.ati_get_face(self.h, mb, which, nn, _dp_of(out)))
        return out.reshape(-1, nbs)

    def get_time(self):
        t = AtiTime()
        self._chk(self.L.ati_get_time(self.h, ctypes.byref(t)))
        return t.as_tuple()

    def set_time(self, tup):
        t = AtiTime(*tup)
        self._chk(self.L.ati_set_time(self.h, ctypes.byref(t)))

    # -- the reference's procedures
    def mpigo(self, nt, nrt, n45):
        self._chk(self.L.ati_mpigo(self.h, nt, nrt, n45))

    def deriv(self, nn, nz, m):
        self._chk(self.L.ati_deriv(self.h, nn, nz, m))

    def filte(self, nn, nz):
        self._chk(self.L.ati_filte(self.h, nn, nz))

    def filter_step(self):
        self._chk(self.L.ati_filter_step(self.h))

    def rk_stage(self, nk):
        self._chk(self.L.ati_rk_stage(self.h, nk))

    def step(self, nsteps=1):
        return self._chk(self.L.ati_step(self.h, nsteps))

    def turbulence_modes(self, cs=0):
        """(nmodes, 8) float32 table: k_x, k_y, k_z, s_x, s_y, s_z, a, psi."""
        n = ctypes.c_int32()
        self._chk(self.L.ati_turbulence_modes(self.h, cs, None, ctypes.byref(n)))
        out = np.empty((n.value, 8), dtype=np.float32)
        self._chk(self.L.ati_turbulence_modes(self.h, cs, out.ctypes.data_as(ctypes.c_void_p), ctypes.byref(n)))
        return out

    def turbulence_sample(self, xyz, t, cs=0):
        """Inflow-turbulence velocity (3, n) at points xyz (3, n) and time t."""
        a = np.ascontiguousarray(xyz, dtype=np.float64)
        n = a.shape[1]
        v = np.empty((3, n))
        self._chk(self.L.ati_turbulence_sample(self.h, cs, float(t), n, _dp_of(a), _dp_of(v)))
        return v

    def tiles(self):
        """(xi, eta, zeta lines per CTA, points per pointwise tile) chosen at init."""
        t = (ctypes.c_int32 * 4)()
        self._chk(self.L.ati_tiles(self.h, t))
        return tuple(t)

    def set_tiles(self, eta=0, zeta=0, points=0):
        """Pin the eta/zeta lines per CTA and points per tile (0 keeps the current one)."""
        t = (ctypes.c_int32 * 4)(0, eta, zeta, points)
        self._chk(self.L.ati_set_tiles(self.h, t))

    def set_tuning(self, enable):
        """Before init: time tile candidates at init (the default) or run on the default tiles."""
        self._chk(self.L.ati_set_tuning(self.h, 1 if enable else 0))

    def tile_plan(self):
        """The handle's whole tile choice (ATI_TILE_PLAN entries), to reuse on a handle of the same shapes."""
        t = (ctypes.c_int32 * TILE_PLAN)()
        self._chk(self.L.ati_get_tile_plan(self.h, t))
        return tuple(t)

    def set_tile_plan(self, plan):
        """Apply a tile plan taken from tile_plan() (results do not depend on it)."""
        t = (ctypes.c_int32 * TILE_PLAN)(*plan)
        self._chk(self.L.ati_set_tile_plan(self.h, t))

    def set_options(self, tma=True, fused_faces=False, paired_lines=True, stress_at_point=True, dense_zeta=False):
        """Kernel options (the library's defaults; results do not depend on them, except dense_zeta's by FP32
        rounding): TMA staging of the mixed path's segmented eta/zeta sweeps, fused face chains, paired-line
        segmented derivative sweeps, the FP64 path's viscous fluxes with the stresses at the point, the mixed path's
        zeta derivatives as dense products.  Returns the options in effect as a dict."""
        a = ctypes.c_int32()
        flags = ((OPT_TMA if tma else 0) | (OPT_FUSED_FACES if fused_faces else 0)
                 | (OPT_PAIRED_LINES if paired_lines else 0) | (OPT_STRESS_AT_POINT if stress_at_point else 0)
                 | (OPT_DENSE_ZETA if dense_zeta else 0))
        self._chk(self.L.ati_set_options(self.h, flags, ctypes.byref(a)))
        v = a.value
        return {"tma_eta": bool(v & OPT_TMA_ETA), "tma_zeta": bool(v & OPT_TMA_ZETA),
                "fused_faces": bool(v & OPT_FUSED_FACES), "paired_lines": bool(v & OPT_PAIRED_LINES),
                "stress_at_point": bool(v & OPT_STRESS_AT_POINT), "dense_zeta": bool(v & OPT_DENSE_ZETA)}

    def set_spin_limit(self, polls):
        """Polls a device-side barrier wait may take before it gives up (0: the default)."""
        self._chk(self.L.ati_set_spin_limit(self.h, int(polls)))

    def jacobian_sign(self):
        """Per block: bit 0 some J > 0, bit 1 some J < 0, bit 2 J zero or not finite."""
        f = (ctypes.c_int32 * len(self.dims))()
        self._chk(self.L.ati_jacobian_sign(self.h, f))
        return list(f)

    def folded_blocks(self):
        return [b for b, f in enumerate(self.jacobian_sign()) if f not in (1, 2)]

    def step_async(self, nsteps=1):
        """Issue nsteps on the case's stream without waiting."""
        self._chk(self.L.ati_step_async(self.h, nsteps))

    def idle(self):
        v = ctypes.c_int()
        self._chk(self.L.ati_query(self.h, ctypes.byref(v)))
        return bool(v.value)

    def check(self):
        """Wait for the issued steps; raise if the state blew up."""
        self._chk(self.L.ati_check(self.h))

    def synchronize(self):
        self._chk(self.L.ati_synchronize(self.h))

    def set_wait_timeout(self, seconds):
        """Bound the host waits of synchronize / step / check (0: no limit)."""
        self._chk(self.L.ati_set_wait_timeout(self.h, float(seconds)))

    def profile(self, enable=True):
        """Bracket every launch with CUDA events on the case's stream."""
        self._chk(self.L.ati_profile_enable(self.h, 1 if enable else 0))

    def profile_read(self):
        """{kernel class: (milliseconds, launches)} since profiling was enabled."""
        n = len(KERNEL_CLASSES)
        ms = np.zeros(n)
        cnt = (ctypes.c_int64 * n)()
        self._chk(self.L.ati_profile_read(self.h, n, _dp_of(ms), cnt))
        return {k: (float(ms[i]), int(cnt[i])) for i, k in enumerate(KERNEL_CLASSES)}

    def launch_count(self):
        v = ctypes.c_int64()
        self._chk(self.L.ati_launch_count(self.h, ctypes.byref(v)))
        return v.value

    def stream(self):
        """The case's cudaStream_t as an integer handle."""
        return self.L.ati_stream(self.h)

    def forces(self):
        out = np.zeros(2)
        self._chk(self.L.ati_forces(self.h, _dp_of(out)))
        return out

    # -- outputs and files
    def cp(self, mb):
        """Pressure coefficient of the current state (getCp, src/rptPost.f90:1456-1465)."""
        return self.get_field(mb, F_CP)[0]

    def frame(self):
        """(umf[3], aoa in degrees) of the current time."""
        u = np.zeros(3)
        a = ctypes.c_double()
        self._chk(self.L.ati_get_frame(self.h, _dp_of(u), ctypes.byref(a)))
        return u, a.value

    def wall_probe(self, capacity):
        """Record the mid-span wall pressure every step (capacity records, 0 = off)."""
        self._chk(self.L.ati_wall_probe_enable(self.h, int(capacity)))

    def wall_probe_read(self):
        """(times[nrec], p[nrec, npts]) of the recorded steps, oldest first."""
        nr, npt = ctypes.c_int64(), ctypes.c_int64()
        self._chk(self.L.ati_wall_probe_read(self.h, None, None, ctypes.byref(nr), ctypes.byref(npt)))
        p = np.empty((nr.value, npt.value))
        t = np.empty(nr.value)
        self._chk(self.L.ati_wall_probe_read(self.h, _dp_of(p), _dp_of(t), ctypes.byref(nr), ctypes.byref(npt)))
        return t, p

    def write_restart(self, mb, path):
        self._chk(self.L.ati_write_restart(self.h, mb, os.fsencode(path)))

    def read_restart(self, mb, path):
        self._chk(self.L.ati_read_restart(self.h, mb, os.fsencode(path)))

    def write_plot3d_grid(self, path):
        self._chk(self.L.ati_write_plot3d_grid(self.h, os.fsencode(path)))

    def write_plot3d_solution(self, path):
        self._chk(self.L.ati_write_plot3d_solution(self.h, os.fsencode(path)))


class Batch(Case):
    """Several independent cases in one handle (ati_create_batch): one launch
    per kernel and one CUDA graph per step cover every case.  Blocks are
    numbered across the batch (case c owns blocks 6c..6c+5); ``block(c, mb)``
    maps a case's own block number."""

    def __init__(self, cfgs, lib_path=LIB_PATH):
        self.L = load_library(lib_path)
        self.cfgs = list(cfgs)
        self.cfg = self.cfgs[0]
        arr = (type(self.cfg.to_c()) * len(self.cfgs))(*[c.to_c() for c in self.cfgs])
        self._c = arr
        h = ctypes.c_void_p()
        rc = self.L.ati_create_batch(arr, len(self.cfgs), ctypes.byref(h))
        if rc:
            raise AtiError(rc, self.L.ati_last_error(None).decode())
        self.h = h
        self._dims(sum(c.nblocks for c in self.cfgs))

    @property
    def ncase(self):
        return len(self.cfgs)

    def block(self, cs, mb):
        first, n = ctypes.c_int(), ctypes.c_int()
        self._chk(self.L.ati_case_blocks(self.h, cs, ctypes.byref(first), ctypes.byref(n)))
        assert 0 <= mb < n.value
        return first.value + mb

    def case_state(self, cs):
        return [self.get_state(self.block(cs, mb)) for mb in range(self.cfgs[cs].nblocks)]

    def case_time(self, cs):
        t = AtiTime()
        self._chk(self.L.ati_case_time(self.h, cs, ctypes.byref(t)))
        return t.as_tuple()

    def case_check(self, cs):
        """Raise AtiError (ATI_ENONFINITE) if case cs of the batch has failed."""
        self._chk(self.L.ati_case_check(self.h, cs))

    def case_forces(self, cs):
        out = np.zeros(2)
        self._chk(self.L.ati_case_forces(self.h, cs, _dp_of(out)))
        return out


def setup_batch(cfgs, grids=None):
    """Create a batch, upload every case's aerofoil grid and run the set-up."""
    from .grid import aerofoil_grid
    b = Batch(cfgs)
    for cs, cfg in enumerate(b.cfgs):
        g = aerofoil_grid(cfg) if grids is None else grids[cs]
        for mb in range(cfg.nblocks):
            b.set_grid(b.block(cs, mb), g[mb])
    b.init()
    return b


def probe_fma_tflops(fp64=True):
    """Measured FMA throughput of this GPU (TFLOP/s)."""
    L = load_library()
    v = ctypes.c_double()
    rc = L.ati_probe_fma_tflops(1 if fp64 else 0, ctypes.byref(v))
    if rc:
        raise AtiError(rc, "ati_probe_fma_tflops failed")
    return v.value


def dense_zeta_operator(cfg: CaseConfig, blk):
    """The L x L FP64 operator of block blk's zeta derivative that the dense zeta option applies (host only)."""
    L = load_library()
    c = cfg.to_c()
    m = np.zeros(64 * 64)
    n = ctypes.c_int32()
    rc = L.ati_dense_zeta_operator(ctypes.byref(c), blk, m.ctypes.data_as(_dp), ctypes.byref(n))
    if rc:
        raise AtiError(rc, L.ati_last_error(None).decode())
    return m[:n.value * n.value].reshape(n.value, n.value).copy()


def setup_case(cfg: CaseConfig, grid=None, cls=Case):
    """Create a case, upload the aerofoil grid and run the set-up."""
    from .grid import aerofoil_grid
    c = cls(cfg)
    g = aerofoil_grid(cfg) if grid is None else grid
    for mb in range(cfg.nblocks):
        c.set_grid(mb, g[mb])
    c.init()
    return c
