"""Error of the mixed-precision path (ATI_MIXED) against the FP64 path on one
case, for every output the solver produces:

  field L2      relative L2 per conserved variable and of the whole state
  surface Cp    (p - p_inf) 2 / M^2 on the mid-span wall lines (getCp,
                src/rptPost.f90:1456-1465)
  Cl / Cd       the clpost force coefficients (src/rpt.f90:1017-1056)
  wall PSD      power spectral density of the wall-pressure time series
                recorded every step (no counterpart in the reference)

    python -m tandemproject_gb300.accuracy --preset naca0012_25m --steps 1000 [--dense-zeta]

Both runs start from the same grid and initial state and take the same steps;
the FP64 path itself matches the CPU restatement of the reference to ~1e-14.
"""
import argparse
import json
import time

import numpy as np


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def wall_psd(t, p):
    """One-sided power spectral density of the wall pressure, averaged over the
    wall points: p[r, i] at times t[r] (the CFL time step varies, so each
    point's series is first resampled linearly onto a uniform grid of the same
    length), mean removed, Hann window.  Normalised so that the sum of psd * df
    over the returned frequencies equals the variance of the windowed series
    (a sinusoid of amplitude A gives A^2 / 2).  Returns (freq, psd)."""
    n = len(t)
    tu = np.linspace(t[0], t[-1], n)
    pu = np.stack([np.interp(tu, t, p[:, i]) for i in range(p.shape[1])], axis=1)
    pu = pu - pu.mean(axis=0)
    w = np.hanning(n)[:, None]
    spec = np.abs(np.fft.rfft(pu * w, axis=0)) ** 2
    # one-sided: every bin but zero frequency (and Nyquist, for even n) stands for its negative twin too
    spec[1:n - n // 2] *= 2.0
    dtu = (tu[-1] - tu[0]) / max(n - 1, 1)
    freq = np.fft.rfftfreq(n, dtu)
    return freq, spec.mean(axis=1) * dtu / (w ** 2).sum()


def compare(cfg, steps, probe=True, log=print, dense_zeta=False):
    from .config import FP64, MIXED
    from .grid import aerofoil_grid
    from .solver import setup_case
    grid = aerofoil_grid(cfg)
    out = {"steps": steps, "points": cfg.npoints}
    runs = {}
    for name, prec in (("fp64", FP64), ("mixed", MIXED)):
        c = setup_case(cfg.replace(precision=prec), grid=grid)
        if dense_zeta and prec == MIXED:
            out["dense_zeta"] = c.set_options(dense_zeta=True)["dense_zeta"]
        if probe:
            c.wall_probe(steps)
        t0 = time.time()
        c.step(steps)
        c.synchronize()
        runs[name] = c
        log(f"{name}: {steps} steps in {time.time() - t0:.1f} s")
    d, m = runs["fp64"], runs["mixed"]
    num, den = np.zeros(5), np.zeros(5)
    for mb in range(cfg.nblocks):
        qd, qm = d.get_state(mb), m.get_state(mb)
        num += np.sum((qm - qd) ** 2, axis=1)
        den += np.sum(qd ** 2, axis=1)
    whole = float(np.sqrt(num.sum() / den.sum()))
    mom = float(np.sqrt(num[1:4].sum() / den[1:4].sum()))
    out["field_rel_l2"] = {"rho": float(np.sqrt(num[0] / den[0])), "momentum": mom,
                           "rhoE": float(np.sqrt(num[4] / den[4])), "whole_state": whole}
    fd, fm = d.forces(), m.forces()
    out["forces"] = {"fp64": fd.tolist(), "mixed": fm.tolist(),
                     "rel_err": [float(abs(fm[i] - fd[i]) / max(abs(fd[i]), 1e-300)) for i in range(2)]}
    if probe:
        td, pd = d.wall_probe_read()
        tm, pm = m.wall_probe_read()
        mach2 = cfg.mach ** 2
        cpd, cpm = (pd[-1] - 1 / 1.4) * 2 / mach2, (pm[-1] - 1 / 1.4) * 2 / mach2
        out["wall_cp"] = {"rel_l2": rel_l2(cpm, cpd), "max_abs": float(np.max(np.abs(cpm - cpd))),
                          "points": int(cpd.size)}
        fq, sd = wall_psd(td, pd)
        _, sm = wall_psd(tm, pm)
        out["wall_psd"] = {"rel_l2": rel_l2(sm, sd), "bins": int(sd.size),
                           "max_rel_bin_err_above_1e-3_peak": float(np.max(np.abs(sm - sd)[sd > 1e-3 * sd.max()]
                                                                         / sd[sd > 1e-3 * sd.max()]))}
    for c in runs.values():
        c.close()
    return out


def main():
    from .config import PRESETS
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--preset", default="naca0012_0p6m")
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--nsmf", type=int, default=None, help="override the start (0 = the reference deck's ramp)")
    ap.add_argument("--timf", type=float, default=None)
    ap.add_argument("--dense-zeta", action="store_true", help="the mixed run's zeta derivatives as dense products")
    args = ap.parse_args()
    cfg = PRESETS[args.preset]
    kw = {k: v for k, v in (("nsmf", args.nsmf), ("timf", args.timf)) if v is not None}
    cfg = cfg.replace(**kw)
    res = compare(cfg, args.steps, dense_zeta=args.dense_zeta)
    res["preset"] = args.preset
    res["nsmf"], res["timf"] = cfg.nsmf, cfg.timf
    print(json.dumps(res))


if __name__ == "__main__":
    main()
