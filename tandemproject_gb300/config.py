"""Typed configuration of one aerofoil case: the hot-path fields of the
reference's input decks (inputo.dat read at src/Main3D.f90:34-58, inputp.dat
read at src/SingleTurbulence3D.f90:39-62), mirrored as the C struct
``ati_config_t`` of include/ati.h.

Presets name the workloads by what they are:
  naca0012_0p2m  NACA 0012, 6 blocks (49/121/49)x40x13 = 0.23 M points, FP64 (quick checks)
  naca0012_0p6m  NACA 0012, 6 blocks (91/201/91)x40x20 = 0.61 M points, FP64
  naca0012_3p5m  NACA 0012, 6 blocks 256x96x24 = 3.54 M points, FP64 (profiler captures)
  naca0012_8p8m  NACA 0012, 6 blocks 384x120x32 = 8.85 M points, FP64
  naca0012_25m   NACA 0012, 6 blocks 640x200x32 = 24.6 M points, mixed
"""
import ctypes
import dataclasses

MAX_BK = 8
FP64 = 0
MIXED = 1
FP64_STRICT = 2


class AtiConfig(ctypes.Structure):
    """ctypes image of ati_config_t (include/ati.h)."""
    _fields_ = [
        ("bkx", ctypes.c_int32), ("bky", ctypes.c_int32), ("bkz", ctypes.c_int32),
        ("lxibk", ctypes.c_int32 * MAX_BK), ("letbk", ctypes.c_int32 * MAX_BK),
        ("lzebk", ctypes.c_int32 * MAX_BK),
        ("nkrk", ctypes.c_int32), ("nviscous", ctypes.c_int32), ("nsmf", ctypes.c_int32),
        ("les", ctypes.c_int32), ("precision", ctypes.c_int32),
        ("turb_modes", ctypes.c_int32), ("turb_seed", ctypes.c_int32),
        ("reserved_i", ctypes.c_int32 * 5),
        ("reoo", ctypes.c_double), ("tempoo", ctypes.c_double),
        ("amach1", ctypes.c_double), ("amach2", ctypes.c_double), ("amach3", ctypes.c_double),
        ("wtemp", ctypes.c_double), ("cfl", ctypes.c_double), ("timf", ctypes.c_double),
        ("fltk", ctypes.c_double), ("fltkbc", ctypes.c_double), ("dto", ctypes.c_double),
        ("aoa0", ctypes.c_double), ("aoa1", ctypes.c_double), ("tps", ctypes.c_double),
        ("tp", ctypes.c_double),
        ("smago1", ctypes.c_double), ("smago2", ctypes.c_double),
        ("domlen", ctypes.c_double), ("span", ctypes.c_double),
        ("szth1", ctypes.c_double), ("szth2", ctypes.c_double), ("szxt", ctypes.c_double),
        ("szco", ctypes.c_double),
        ("turb_intensity", ctypes.c_double), ("turb_length", ctypes.c_double),
        ("reserved_d", ctypes.c_double * 6),
    ]


class AtiTime(ctypes.Structure):
    """ctypes image of ati_time_t: n, ndt, dt, dts, dte, timo."""
    _fields_ = [("n", ctypes.c_int64), ("ndt", ctypes.c_int64), ("dt", ctypes.c_double),
                ("dts", ctypes.c_double), ("dte", ctypes.c_double), ("timo", ctypes.c_double)]

    def as_tuple(self):
        return (self.n, self.ndt, self.dt, self.dts, self.dte, self.timo)


@dataclasses.dataclass
class CaseConfig:
    """One case.  Sizes are last indices (lxi = points - 1) as in the decks."""
    lxibk: tuple = (90, 200, 90)
    letbk: tuple = (39, 39)
    lzebk: tuple = (19,)
    nkrk: int = 4
    nviscous: int = 1
    nsmf: int = 1
    les: int = 0
    precision: int = FP64
    reoo: float = 4.0e5
    tempoo: float = 273.0
    mach: float = 0.24
    aoa_deg: float = 0.0
    wtemp: float = 1.0
    cfl: float = 0.8
    timf: float = 15.0
    fltk: float = 0.85
    fltkbc: float = 0.85
    dto: float = -1.0
    tp: float = 0.0
    tps: float = 0.0
    aoa1: float = 0.0
    smago1: float = 0.16
    smago2: float = 0.0066
    # grid and sponge (inputp.dat)
    domlen: float = 10.0
    span: float = 0.1
    szth1: float = 2.0
    szth2: float = 2.0
    szxt: float = 4.0
    szco: float = 12.0
    thick: float = 12.0         # NACA 00tt thickness in percent of chord
    smgrid: float = 0.0075
    ximod: float = 0.05
    etamod: float = 0.05
    wlew: float = 0.11
    wlea: float = 0.0
    chord: float = 1.0
    delt_deg: float = 0.0
    # synthetic inflow turbulence (0 intensity: none)
    turb_intensity: float = 0.0  # rms per velocity component / |U_inf|
    turb_length: float = 0.1     # von Karman integral length (chord units)
    turb_modes: int = 2048
    turb_seed: int = 1234

    @property
    def bkx(self):
        return len(self.lxibk)

    @property
    def bky(self):
        return len(self.letbk)

    @property
    def bkz(self):
        return len(self.lzebk)

    def block_dims(self, mb):
        i = mb % self.bkx
        j = (mb // self.bkx) % self.bky
        k = mb // (self.bkx * self.bky)
        return self.lxibk[i], self.letbk[j], self.lzebk[k]

    @property
    def nblocks(self):
        return self.bkx * self.bky * self.bkz

    @property
    def npoints(self):
        n = 0
        for mb in range(self.nblocks):
            a, b, c = self.block_dims(mb)
            n += (a + 1) * (b + 1) * (c + 1)
        return n

    def to_c(self):
        import math
        c = AtiConfig()
        c.bkx, c.bky, c.bkz = self.bkx, self.bky, self.bkz
        for i, v in enumerate(self.lxibk):
            c.lxibk[i] = v
        for i, v in enumerate(self.letbk):
            c.letbk[i] = v
        for i, v in enumerate(self.lzebk):
            c.lzebk[i] = v
        c.nkrk, c.nviscous, c.nsmf, c.les, c.precision = (
            self.nkrk, self.nviscous, self.nsmf, self.les, self.precision)
        c.reoo, c.tempoo = self.reoo, self.tempoo
        a = math.radians(self.aoa_deg)
        # inputo.dat convention: amach1 = M cos(aoa), amach2 = M sin(aoa)
        c.amach1, c.amach2, c.amach3 = self.mach * math.cos(a), self.mach * math.sin(a), 0.0
        c.wtemp, c.cfl, c.timf = self.wtemp, self.cfl, self.timf
        c.fltk, c.fltkbc, c.dto = self.fltk, self.fltkbc, self.dto
        c.aoa0, c.aoa1, c.tps, c.tp = self.aoa_deg, self.aoa1, self.tps, self.tp
        c.smago1, c.smago2 = self.smago1, self.smago2
        c.domlen, c.span = self.domlen, self.span
        c.szth1, c.szth2, c.szxt, c.szco = self.szth1, self.szth2, self.szxt, self.szco
        c.turb_modes = self.turb_modes if self.turb_intensity > 0 else 0
        c.turb_seed, c.turb_intensity, c.turb_length = self.turb_seed, self.turb_intensity, self.turb_length
        return c

    def replace(self, **kw):
        return dataclasses.replace(self, **kw)


PRESETS = {
    "naca0012_0p6m": CaseConfig(),
    # a 228 K-point case whose CPU run takes seconds (smoke checks, quick benches)
    "naca0012_0p2m": CaseConfig(lxibk=(48, 120, 48), letbk=(39, 39), lzebk=(12,)),
    # smgrid scales the near-wall spacing with resolution so that the quintic
    # grid lines of gridf stay monotone (no folded cells) at these sizes
    # the plain-FP64 larger configuration: seeded von Karman inflow turbulence,
    # 2.5 % of U_inf, integral length 0.1 c, 2048 modes from seed 1234
    # (the reference deck's smooth start, nsmf = 0: on this grid the impulsive start diverges between steps 600 and
    # 625, with and without the inflow turbulence, short of the 1000 steps this case runs)
    "naca0012_8p8m": CaseConfig(lxibk=(383, 383, 383), letbk=(119, 119), lzebk=(31,), smgrid=0.0025,
                                turb_intensity=0.025, nsmf=0, timf=1.0),
    # a 3.5 M-point case (2.4 GB FP64 arena, state larger than L2) for profiler captures
    "naca0012_3p5m": CaseConfig(lxibk=(255, 255, 255), letbk=(95, 95), lzebk=(23,), smgrid=0.004),
    "naca0012_25m": CaseConfig(lxibk=(639, 639, 639), letbk=(199, 199), lzebk=(31,), smgrid=0.002,
                               precision=MIXED),
}


def small_case(lxibk=(24, 64, 24), letbk=(16, 16), lzebk=(12,), **kw):
    """A small aerofoil case whose oracle run takes seconds (tests)."""
    return CaseConfig(lxibk=lxibk, letbk=letbk, lzebk=lzebk, **kw)
