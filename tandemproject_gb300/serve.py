"""Serving loop: aerofoil solves arrive over time, are admitted by device-
memory footprint under a budget, stay resident on the GPU while they run, and
leave when their steps are done.  Admission is continuous: a request that
arrives while others are running starts as soon as memory is free, and the
work of all running requests overlaps on the device (one CUDA stream per
case, steps issued in chunks without waiting).

    python -m tandemproject_gb300.serve --requests 16 --step-scale 0.1

Each request's result (final state, forces) is the same as when it runs
alone: cases share nothing on the device.  A request whose state turns
non-finite (ATI_ENONFINITE after one of its chunks: the compact scheme has no
shock capturing, and the upper corner of the parameter ranges can diverge) is
retired as failed, with the steps it had run, and its memory goes to the
others; so is a request whose set-up the library refuses (an error status
from ati_create or ati_init, such as device memory taken by other processes).
The latency percentiles are those of the completed requests.
"""
import argparse
import concurrent.futures as cf
import json
import time

import numpy as np

from .solver import AtiError
from .workloads import fold_free_case, footprint_bytes, relax, serving_requests, valid_grid

ATI_ENONFINITE = 4


def _gpu_case(cfg, grid, plan=None):
    """A case set up on the GPU; with a tile plan of an earlier case of the same block shapes, ati_init does not time
    tile candidates again (results do not depend on tiles)."""
    from .solver import Case
    c = Case(cfg)
    if plan is not None:
        c.set_tuning(False)
    for mb in range(cfg.nblocks):
        c.set_grid(mb, grid[mb])
    c.init()
    if c.folded_blocks():  # the grid folds under the compact metrics: take a relaxed grid of the same size
        c.close()
        _, _, c = fold_free_case(relax(cfg))
        plan = None
    if plan is not None:
        c.set_tile_plan(plan)
    return c


def _params(cfg):
    """The drawn parameters of a request, for the record of a failed one."""
    return {k: getattr(cfg, k) for k in ("mach", "aoa_deg", "thick", "turb_intensity")}


def plan_key(cfg):
    """Cases that share their tile plan: the same numerics and block shapes."""
    return (cfg.precision, cfg.nviscous, cfg.les, tuple(cfg.lxibk), tuple(cfg.letbk), tuple(cfg.lzebk))


class Server:
    def __init__(self, budget_bytes=150 << 30, chunk=10, prefetch=4, keep_state=False, make_case=_gpu_case,
                 make_grid=valid_grid, footprint=footprint_bytes):
        self.budget = budget_bytes
        self.chunk = chunk
        self.prefetch = prefetch
        self.keep_state = keep_state
        self.make_case = make_case
        self.make_grid = make_grid
        self.footprint = footprint
        self.peak_bytes = 0
        self.bound = False  # some request waited for memory (admission held it back)
        self.plans = {}     # tile plans by plan_key: a case of known shapes skips the tile timing at set-up
        self.plan_hits = 0

    def run(self, requests, log=None):
        """Serve the requests (arrival times in seconds from the start);
        return one record per request and the run summary.

        The issuing loop never waits for a case to be set up: host grids are
        built from arrival on (prefetch pool), and an admitted case is created
        and initialised (device arrays, metrics, tile timing) on a set-up
        thread while the loop keeps issuing steps to the running cases.  Its
        memory counts against the budget from admission on.  The tile timing
        runs once per block shape: later cases of the same shapes reuse its
        plan (plan_key)."""
        pending = sorted(requests, key=lambda r: r.arrival)
        waiting, starting, active, done, failed = [], [], [], [], []
        used = 0
        grids = {}
        pool = cf.ThreadPoolExecutor(max_workers=self.prefetch)
        setup = cf.ThreadPoolExecutor(max_workers=1)
        t0 = time.perf_counter()
        now = lambda: time.perf_counter() - t0

        def create(r):
            cfg, grid = grids.pop(r.rid).result()
            key = plan_key(cfg)
            plan = self.plans.get(key)
            if plan is None:
                c = self.make_case(cfg, grid)
                if hasattr(c, "tile_plan"):
                    self.plans[key] = c.tile_plan()
            else:
                c = self.make_case(cfg, grid, plan=plan)
                self.plan_hits += 1
            return cfg, c

        while pending or waiting or starting or active:
            t = now()
            while pending and pending[0].arrival <= t:
                r = pending.pop(0)
                waiting.append(r)
                grids[r.rid] = pool.submit(self.make_grid, r.cfg)  # host-side grid, ahead of admission
            # admit in arrival order while the footprint fits; the set-up runs off the issuing loop
            while waiting:
                r = waiting[0]
                fp = self.footprint(r.cfg)
                if used + fp > self.budget and (active or starting):
                    self.bound = True
                    break
                waiting.pop(0)
                used += fp
                self.peak_bytes = max(self.peak_bytes, used)
                starting.append({"req": r, "fp": fp, "admitted": now(), "job": setup.submit(create, r)})
                if log:
                    log(f"t={now():7.2f}s admit #{r.rid} {r.cfg.npoints / 1e6:.2f} M pts x {r.steps} steps, "
                        f"{used / 2**30:.1f} GiB in use")
            for s in list(starting):
                if s["job"].done():
                    starting.remove(s)
                    try:
                        cfg, c = s["job"].result()
                    except AtiError as err:  # the library refused the case (device memory, configuration)
                        r = s["req"]
                        used -= s["fp"]
                        failed.append({"id": r.rid, "points": r.cfg.npoints, "steps": r.steps, "steps_run": 0,
                                       "arrival": r.arrival, "failed_at": now(), "error": str(err),
                                       "params": _params(r.cfg)})
                        if log:
                            log(f"t={now():7.2f}s FAILED #{r.rid} at set-up: {err}")
                        continue
                    active.append({"req": s["req"], "case": c, "left": s["req"].steps, "fp": s["fp"],
                                   "admitted": s["admitted"], "started": now(), "npts": cfg.npoints,
                                   "issued": 0, "checked": 0})
            # a case whose last chunk is done: its status (a diverged request is retired as failed)
            for a in list(active):
                if a["issued"] > a["checked"] and a["case"].idle():
                    try:
                        a["case"].check()
                        a["checked"] = a["issued"]
                    except Exception as err:
                        if getattr(err, "code", None) != ATI_ENONFINITE:
                            raise
                        r = a["req"]
                        rec = {"id": r.rid, "points": a["npts"], "steps": r.steps, "steps_run": a["issued"],
                               "arrival": r.arrival, "failed_at": now(), "error": str(err),
                               "params": _params(r.cfg)}
                        a["case"].close()
                        used -= a["fp"]
                        active.remove(a)
                        failed.append(rec)
                        if log:
                            log(f"t={now():7.2f}s FAILED #{r.rid} after {a['issued']} of {r.steps} steps: {err}")
            # one chunk of steps for every running case, issued without waiting
            for a in active:
                if a["left"] > 0 and a["case"].idle() and a["checked"] == a["issued"]:
                    k = min(self.chunk, a["left"])
                    a["case"].step_async(k)
                    a["left"] -= k
                    a["issued"] += k
            # retire finished cases
            for a in list(active):
                if a["left"] == 0 and a["case"].idle() and a["checked"] == a["issued"]:
                    c = a["case"]
                    rec = {"id": a["req"].rid, "points": a["npts"], "steps": a["req"].steps,
                           "arrival": a["req"].arrival, "admitted": a["admitted"], "started": a["started"],
                           "done": now(), "forces": c.forces().tolist()}
                    if self.keep_state:
                        rec["state"] = [c.get_state(mb) for mb in range(c.cfg.nblocks)]
                    rec["latency"] = rec["done"] - rec["arrival"]
                    c.close()
                    used -= a["fp"]
                    active.remove(a)
                    done.append(rec)
                    if log:
                        log(f"t={now():7.2f}s done  #{rec['id']} latency {rec['latency']:.2f} s")
            if not pending and not waiting and (active or starting):
                time.sleep(0.0005)
            elif pending and not waiting and not active and not starting:
                time.sleep(max(0.0, min(pending[0].arrival - now(), 0.05)))
        pool.shutdown()
        setup.shutdown()
        makespan = now()
        lat = np.array([d["latency"] for d in done] or [np.nan])
        wait = np.array([d["admitted"] - d["arrival"] for d in done] or [np.nan])
        work = sum(d["points"] * 4 * d["steps"] for d in done)
        summary = {"requests": len(done), "makespan_s": makespan,
                   "latency_s": {"p50": float(np.percentile(lat, 50)), "p95": float(np.percentile(lat, 95)),
                                 "p99": float(np.percentile(lat, 99)), "max": float(lat.max())},
                   "admission_wait_s": {"p50": float(np.percentile(wait, 50)), "max": float(wait.max())},
                   "admission_bound": self.bound,
                   "updates_per_s": work / makespan, "peak_resident_gib": self.peak_bytes / 2**30,
                   "tile_plans_reused": self.plan_hits,
                   "failed": len(failed),
                   "failed_requests": [{k: f[k] for k in ("id", "points", "steps", "steps_run", "params")}
                                       for f in failed]}
        return done, summary


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--requests", type=int, default=16)
    ap.add_argument("--rate", type=float, default=4.0)
    ap.add_argument("--seed", type=int, default=99)
    ap.add_argument("--step-scale", type=float, default=1.0)
    ap.add_argument("--budget-gb", type=float, default=150.0)
    ap.add_argument("--precision", type=int, default=1, help="0 = FP64, 1 = mixed")
    ap.add_argument("--chunk", type=int, default=10)
    ap.add_argument("--quiet", action="store_true")
    args = ap.parse_args()
    reqs = serving_requests(args.requests, seed=args.seed, rate=args.rate, precision=args.precision,
                            step_scale=args.step_scale)
    srv = Server(budget_bytes=int(args.budget_gb * 2**30), chunk=args.chunk)
    done, summary = srv.run(reqs, log=None if args.quiet else (lambda m: print(m, flush=True)))
    summary.update({"precision": "mixed" if args.precision == 1 else "fp64", "rate_per_s": args.rate,
                    "seed": args.seed, "step_scale": args.step_scale, "budget_gb": args.budget_gb})
    print(json.dumps(summary))


if __name__ == "__main__":
    main()
