"""Long parity run of the CUDA path against the CPU oracle (a record, not a
collected test): one case stepped on the GPU and on the oracle for many steps,
relative L2 per conserved variable every `--every` steps.

    python tests/parity_long.py --preset naca0012_8p8m --steps 1000 --every 100

The 8.85 M-point preset is the plain FP64 method's case with seeded von
Karman inflow turbulence; with --precision strict the GPU sums the
turbulence modes in FP64 in the oracle's order.  The oracle takes about 1.5 s
a step on 16 host cores.
"""
import argparse
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def main():
    from oracle.oracle import OracleCase, build_modes, get_threads, set_threads
    from tandemproject_gb300.config import FP64, FP64_STRICT, PRESETS
    from tandemproject_gb300.grid import aerofoil_grid
    from tandemproject_gb300.solver import setup_case
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--preset", default="naca0012_8p8m")
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--every", type=int, default=100)
    ap.add_argument("--precision", choices=["fp64", "strict"], default="strict")
    ap.add_argument("--threads", type=int, default=0, help="oracle threads (0: all host cores)")
    args = ap.parse_args()
    if args.threads > 0:
        set_threads(args.threads)
    cfg = PRESETS[args.preset].replace(precision=FP64_STRICT if args.precision == "strict" else FP64)
    grid = aerofoil_grid(cfg)
    gpu = setup_case(cfg, grid=grid)
    orc = OracleCase(cfg)
    for mb in range(cfg.nblocks):
        orc.set_grid(mb, grid[mb])
    orc.init()
    modes = build_modes(cfg)
    if modes.size:
        orc.set_turbulence(modes)
    done = 0
    t_gpu = t_orc = 0.0
    while done < args.steps:
        k = min(args.every, args.steps - done)
        t0 = time.perf_counter()
        gpu.step(k)
        gpu.synchronize()
        t_gpu += time.perf_counter() - t0
        t0 = time.perf_counter()
        rc = orc.step(k)
        t_orc += time.perf_counter() - t0
        done += k
        num, den = np.zeros(5), np.zeros(5)
        for mb in range(cfg.nblocks):
            q, qo = gpu.get_state(mb), orc.get_state(mb)
            num += np.sum((q - qo) ** 2, axis=1)
            den += np.sum(qo ** 2, axis=1)
        den[1:4] = den[1:4].sum()
        e = np.sqrt(num / den)
        tg, to = gpu.get_time(), orc.get_time()
        print(json.dumps({"preset": args.preset, "precision": args.precision, "step": done, "oracle_rc": rc,
                          "rel_l2": {"rho": e[0], "momentum_x": e[1], "momentum_y": e[2], "momentum_z": e[3],
                                     "rhoE": e[4]},
                          "dt_rel": abs(tg[2] - to[2]) / abs(to[2]) if to[2] else 0.0,
                          "gpu_s": round(t_gpu, 2), "oracle_s": round(t_orc, 1),
                          "oracle_threads": get_threads(), "turbulence_modes": int(modes.shape[0])}), flush=True)


if __name__ == "__main__":
    main()
