"""Seeded synthetic workloads of many aerofoil cases: the batched form (many
independent cases stepped together) and the serving form (requests arriving
over time).  Parameters follow the case ranges of those forms: NACA 00tt
thickness t in U[8,18] %, angle of attack in U[0,8] deg, Mach in U[0.2,0.4],
inflow turbulence intensity in U[0,5] % (von Karman, 2048 modes, integral
length 0.1 chord), uneven grid sizes, spanwise 16-48 points.  Every case
starts from rest with the reference deck's smooth frame ramp (nsmf = 0) over
one time unit: an impulsive start on these grids diverges within a few
hundred steps for the thicker sections and higher Mach numbers.
"""
import dataclasses
import math

import numpy as np

from .config import MIXED, CaseConfig


def sized_case(npoints, nz, seed_rng, precision=MIXED, aspect=3.2, nx_min=160, ny_min=56, **kw):
    """A NACA 00tt case of about npoints points: 6 blocks of nx x ny x nz with
    the xi/eta aspect of the reference grid (nx ~ 3.2 ny).  The in-plane grid
    keeps at least nx_min x ny_min points per block (coarser aerofoil grids
    diverge under the compact scheme); small cases give up spanwise points
    instead (nz stays within 16-48)."""
    ny = max(ny_min, int(round(math.sqrt(npoints / (6.0 * nz * aspect)))))
    nx = int(round(npoints / (6.0 * ny * nz)))
    if nx < nx_min:
        nx = nx_min
        nz = int(min(48, max(16, round(npoints / (6.0 * nx * ny)))))
    smgrid = min(0.0075, max(0.002, 1.0 / nx))
    kw.setdefault("nsmf", 0)
    kw.setdefault("timf", 1.0)
    return CaseConfig(lxibk=(nx - 1,) * 3, letbk=(ny - 1,) * 2, lzebk=(nz - 1,), smgrid=smgrid, precision=precision,
                      **kw)


def valid_grid(cfg, tries=4):
    """Return (cfg, grid) with a fold-free grid, tightening the wall spacing if needed."""
    from .grid import aerofoil_grid, min_cell_jacobian
    for _ in range(tries):
        g = aerofoil_grid(cfg)
        j = min_cell_jacobian(g)
        if all(a < 0 and b < 0 for a, b in j) or all(a > 0 and b > 0 for a, b in j):
            return cfg, g
        cfg = cfg.replace(smgrid=cfg.smgrid * 0.7)
    raise ValueError(f"no fold-free grid for {cfg}")


def relax(cfg):
    """The same case with about the same point count and 25 % more eta lines
    (a coarse eta resolution is what folds the wake-line cells); xi sizes
    shrink in proportion."""
    f = 1.25
    let = tuple(int(round((v + 1) * f)) - 1 for v in cfg.letbk)
    lxi = tuple(max(23, int(round((v + 1) / f)) - 1) for v in cfg.lxibk)
    return cfg.replace(lxibk=lxi, letbk=let, smgrid=min(0.0075, max(0.002, 1.0 / (lxi[1] + 1))))


def fold_free_case(cfg, tries=4):
    """Set the case up on the GPU and check that its Jacobian keeps one sign in
    every block (ati_jacobian_sign); relax the grid and retry if not.
    Returns (cfg, grid, case) with the case initialised."""
    from .solver import setup_case
    for _ in range(tries):
        cfg, g = valid_grid(cfg)
        c = setup_case(cfg, grid=g)
        if not c.folded_blocks():
            return cfg, g, c
        c.close()
        cfg = relax(cfg)
    raise ValueError(f"no fold-free grid for {cfg}")


def _params(rng, index, seed):
    p = dict(thick=float(rng.uniform(8.0, 18.0)), aoa_deg=float(rng.uniform(0.0, 8.0)),
             mach=float(rng.uniform(0.2, 0.4)))
    tu = float(rng.uniform(0.0, 5.0))
    # the turbulence seed is derived, not drawn, so the size and step draws keep their sequence
    p.update(turb_intensity=tu / 100.0, turb_length=0.1, turb_modes=2048, turb_seed=1000 * seed + index)
    return p, tu


def batch_cases(n=16, seed=7, precision=MIXED, nmin=1.0e6, nmax=6.0e6):
    """n cases with sizes spread unevenly over [nmin, nmax] points."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        p, tu = _params(rng, i, seed)
        npts = float(rng.uniform(nmin, nmax))
        nz = int(rng.integers(16, 49))
        out.append((sized_case(npts, nz, rng, precision=precision, **p), {"turbulence_intensity_pct": tu}))
    return out


@dataclasses.dataclass
class Request:
    rid: int
    cfg: CaseConfig
    steps: int
    arrival: float
    meta: dict


def serving_requests(n, seed=99, rate=4.0, nmin=0.5e6, nmax=20.0e6, smin=200, smax=2000, precision=MIXED,
                     step_scale=1.0):
    """n requests with Poisson arrivals (rate per second), sizes log-uniform in
    [nmin, nmax] points, step counts uniform in [smin, smax] (times step_scale)."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for i in range(n):
        t += float(rng.exponential(1.0 / rate))
        p, tu = _params(rng, i, seed)
        npts = float(math.exp(rng.uniform(math.log(nmin), math.log(nmax))))
        nz = int(rng.integers(16, 49))
        steps = max(3, int(round(int(rng.integers(smin, smax + 1)) * step_scale)))
        out.append(Request(i, sized_case(npts, nz, rng, precision=precision, **p), steps, t,
                           {"turbulence_intensity_pct": tu, "target_points": npts}))
    return out


def footprint_bytes(cfg):
    """Device memory of one case handle: the FP64 arena (93 planes of 8 B) and,
    for the mixed path, the FP32 planes (77 of 4 B), plus face buffers."""
    n = cfg.npoints
    per = 93 * 8 + (77 * 4 if cfg.precision == MIXED else 0)
    return int(n * per * 1.03) + (64 << 20)
