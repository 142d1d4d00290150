"""Benchmark: grid-point-stage updates/s of the ATI3D per-RK-stage hot path.

A step is one full time step of the solver (per-step filter + 4 RK stages,
src/Main3D.f90:552-965) over every block of one aerofoil case resident in HBM.
The default workload is the 8.85 M-point NACA 0012 case in FP64
(6 blocks 384x120x32, the reference's plain-FP64 larger-size configuration);
grid-point-stage updates/s = points * 4 * steps / time.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Our arm prints one JSON line with the device-timed value (CUDA events on the
solver's own stream), the end-to-end value through the C ABI with host
buffers (pinned host -> device copy of the state and device -> host copy of
the result inside every step), the roofline of the dominant kernel measured
live from profiled launches, a CPU baseline (the CPU restatement of the
reference, all host cores, bounded sample), clocks sampled during the timed
region and the number of kernel launches.  Sub-objects report the mixed-
precision path on its own configuration, the 24.6 M-point case, beside an
FP64 run of the same case ("mixed"); 16 independent cases in one batched
handle for 500 steps ("batch"); and serving runs of the FP64 and the mixed
path with Poisson arrivals and p50/p95/p99 latency ("serving").  Under torchrun every rank runs an
independent replica of the case (the path has no exchange between GPUs);
value is the sum over ranks divided by the slowest rank's time.

--impl reference times the CPU restatement of the reference (the Fortran
reference has no compiler on this system) with all host threads on the same
workload, on rank 0 only.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "grid-pt-stage updates/s FP64 vs mixed (rel L2 ≤1e-6); p50/p99 solve latency"
UNIT = "grid-pt-stage updates/s"
L2_BYTES = 129 * 2 ** 20

# algorithmic work per unit of a line-sweep launch, a unit being one point of
# one field (one input value read, one output value written; flops of the
# 7-point RHS + forward + backward pass).  A launch sweeps every line of one
# direction over all blocks for several fields at once.
SWEEP_BYTES = {"deriv": 16, "filter": 16}
SWEEP_FLOPS = {"deriv": 17, "filter": 22}
# the mixed path: FP32 derivative sweeps (4 B in, 4 B out); the filter reads
# and writes the FP64 state
SWEEP_BYTES_MIXED = {"deriv": 8, "filter": 16}
# algorithmic bytes per point of the mixed path's pointwise kernels: the viscous
# flux kernel k_flux_staged reads the FP64 state (40 B), the FP32
# metrics (36 B), the twelve derivative planes of u, v, w, T (48 B), Jacobian,
# viscosity, velocity and pressure (24 B) and writes 15 FP32 fluxes (60 B); it
# takes the stresses at the point, so no stress plane is written or read
POINTWISE_BYTES_MIXED = {"flux": 208}
# fields swept per direction per time step: 4 viscous gradients + 5 fluxes in
# each of the 4 stages, or the 5 variables once for the filter
FIELD_SWEEPS_PER_STEP = {"deriv": 4 * (4 + 5), "filter": 5}
# DRAM bytes per unit of the FP64 xi derivative sweep measured with ncu
# (dram__bytes_read.sum + dram__bytes_write.sum of one 5-field launch on the
# 3.54 M-point case: 489.35 MB for 17.69 M units); the kernel streams, so the
# traffic of a launch scales with the units it processes
SWEEP_TRAFFIC_PER_UNIT = {"deriv_xi": 489.35e6 / (5 * 3538944)}
# DRAM bytes per point of k_flux_visc measured with ncu (dram__bytes_read.sum + dram__bytes_write.sum of one launch
# on the 3.54 M-point case: 906.4 + 395.5 MB); the kernel streams, so the traffic scales with the points
FLUX_TRAFFIC_PER_POINT = (906.36e6 + 395.46e6) / 3538944
# algorithmic bytes per point of the FP64 fast path's viscous flux kernel k_flux_visc (the stresses of k_visc taken
# at the point): it reads the metrics (72 B), the twelve derivative planes of u, v, w, T (96 B), Jacobian and
# viscosity (16 B), velocity (24 B), pressure (8 B) and the state (40 B), and writes 15 fluxes (120 B)
FLUX_BYTES_FP64 = 376
# its FP64 flops per point (an FMA counts two), from ncu's opcode counts of one launch on the 3.54 M-point case:
# 81 DFMA, 42 DMUL and 15 DADD a point
FLUX_FLOPS_FP64 = 219
# canonical bytes per grid-point-stage of the whole stage: 141 FP64 words, or
# the mixed data flow with FP32 intermediates and FP64 state/metrics
STAGE_BYTES_FP64 = 1128
STAGE_BYTES_MIXED = 728


def max_over_ranks(t, dist):
    """The largest of every rank's t (the job's time is its slowest rank's): an all-reduce over the process group,
    on the GPU under NCCL, on the host under gloo; t itself without a group."""
    if dist is None:
        return t
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    tt = torch.tensor([float(t)], dtype=torch.float64, device=dev)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    return float(tt.item())


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.idx = gpu_index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL,
                                         text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        rows = [r for r in self.rows if len(r) >= 9]
        idxs = sorted({r[0] for r in rows})
        if len(idxs) > 1:
            rows = [r for r in rows if r[0] == str(self.idx)]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def _oracle_turbulence(o, cfg):
    """The case's inflow turbulence on the oracle (the same mode table, summed in FP64); a note for the sample."""
    from oracle import oracle as orc
    modes = orc.build_modes(cfg)
    if not modes.size:
        return ""
    o.set_turbulence(modes)
    return f"; with the same inflow turbulence ({modes.shape[0]} modes, summed in FP64)"


def _oracle_flags():
    from oracle import build as ob
    return ob.CFLAGS


def cpu_baseline(cfg, grid, sample_steps=10, warm_steps=2):
    """The CPU restatement of the reference, all host threads, on the same case: a bounded sample of ten steps
    (about 15-20 s on 16 cores) after two warm-up steps, so that it holds one of the turbulence evaluations that
    come every ten steps, as the timed GPU steps do."""
    from oracle import oracle as orc
    o = orc.OracleCase(cfg)
    for mb in range(cfg.nblocks):
        o.set_grid(mb, grid[mb])
    o.init()
    turb = _oracle_turbulence(o, cfg)
    o.step(warm_steps)
    t0 = time.perf_counter()
    o.step(sample_steps)
    dt = time.perf_counter() - t0
    cores = orc.get_threads()
    o.close()
    return {"value": cfg.npoints * cfg.nkrk * sample_steps / dt, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{sample_steps} time steps ({sample_steps * cfg.nkrk} RK stages) of the full "
                      f"{cfg.npoints}-point case after {warm_steps} warm-up steps, CPU restatement (oracle/), "
                      f"OpenMP over lines, {cores} threads, gcc {' '.join(_oracle_flags())}{turb}"}


def run_reference(args, cfg, grid):
    """--impl reference: the CPU restatement timed alone (rank 0 only)."""
    from oracle import oracle as orc
    o = orc.OracleCase(cfg)
    for mb in range(cfg.nblocks):
        o.set_grid(mb, grid[mb])
    o.init()
    turb = _oracle_turbulence(o, cfg)
    t0 = time.perf_counter()
    o.step(args.warmup)
    t_warm = (time.perf_counter() - t0) / max(args.warmup, 1)
    # bound the timed sample to about two minutes of CPU work
    k = args.steps
    if t_warm * k > 120.0:
        k = max(1, int(120.0 / max(t_warm, 1e-9)))
    t0 = time.perf_counter()
    o.step(k)
    dt = time.perf_counter() - t0
    cores = orc.get_threads()
    value = cfg.npoints * cfg.nkrk * k / dt
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": k, "warmup": args.warmup,
            "ms_per_step": dt / k * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic: NACA 0012 grid from the reference's grid generator, uniform "
                                    "freestream initial state",
            "impl": "reference",
            "config": {"workload": args.preset, "points": cfg.npoints},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"{k} time steps of the full case after {args.warmup} warm-up steps "
                                       f"(CPU restatement of the reference, gcc {' '.join(_oracle_flags())}; the "
                                       f"Fortran reference has no compiler here){turb}"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    o.close()
    return line


def batch_leg(args, barrier):
    """The batched form: 16 independent cases (seed 7; NACA 00tt, t in 8-18 %, AoA 0-8 deg, M 0.2-0.4, inflow
    turbulence 0-5 %, 1-6 M points each, spanwise 16-48) in one handle, mixed precision, args.batch_steps steps
    (500, the batched configuration's step count); against the same cases run one handle at a time for
    args.batch_seq_steps steps each (the per-step time is steady, so fewer steps measure it)."""
    import torch
    from tandemproject_gb300.solver import Case, setup_batch
    from tandemproject_gb300.workloads import batch_cases, fold_free_case
    cases = batch_cases(16, seed=7)
    cg = []
    for c, _ in cases:  # fold-free grids (checked on the GPU one case at a time)
        cfg, g, h = fold_free_case(c)
        h.close()
        cg.append((cfg, g))
    cfgs = [c for c, _ in cg]
    npts = sum(c.npoints for c in cfgs)
    b = setup_batch(cfgs, grids=[g for _, g in cg])
    st = torch.cuda.ExternalStream(b.stream())
    b.step(args.warmup)
    barrier()
    l0 = b.launch_count()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    b.step(args.batch_steps)
    e1.record(st)
    barrier()
    t_b = e0.elapsed_time(e1) / 1e3
    launches = b.launch_count() - l0
    for cs in range(len(cfgs)):
        b.case_check(cs)
    b.close()
    # the same cases, one handle at a time
    t_seq, ks = 0.0, args.batch_seq_steps
    for cfg, (_, g) in zip(cfgs, cg):
        c = Case(cfg)
        for mb in range(cfg.nblocks):
            c.set_grid(mb, g[mb])
        c.init()
        c.step(args.warmup)
        s1 = torch.cuda.ExternalStream(c.stream())
        barrier()
        a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a0.record(s1)
        c.step(ks)
        a1.record(s1)
        barrier()
        t_seq += a0.elapsed_time(a1) / 1e3
        c.close()
    v_b = npts * 4 * args.batch_steps / t_b
    v_s = npts * 4 * ks / t_seq
    return {"workload": f"16 cases, seed 7: NACA 00tt t 8-18 %, AoA 0-8 deg, M 0.2-0.4, 1-6 M points (uneven), "
                        f"spanwise 16-48, mixed precision, one handle (ati_create_batch), {args.batch_steps} steps "
                        f"after {args.warmup} warm-up steps",
            "points": npts, "steps": args.batch_steps, "value": v_b, "unit": UNIT,
            "ms_per_step": t_b / args.batch_steps * 1e3,
            "gpu_launches_per_step": launches / args.batch_steps,
            "one_case_at_a_time": {"value": v_s, "ms_per_step": t_seq / ks * 1e3, "steps_each": ks},
            "batching_speedup": v_b / v_s,
            "note": "each case has von Karman inflow turbulence of its drawn intensity (2048 modes, L = 0.1 c)"}


def serve_leg(args):
    """The serving form: Poisson arrivals (4/s, seed 99), sizes log-uniform 0.5-20 M points, admitted by device
    footprint, for the FP64 and the mixed path on the same request list.  Step counts U[200,2000] are scaled by
    args.serve_step_scale and the budget is args.serve_budget_gb, both named in the workload: at full step counts
    the run takes many minutes (a separate record), and at a tenth of them a 150 GB budget never binds, so the
    bench's budget is the one under which admission holds requests back."""
    from tandemproject_gb300.config import FP64, MIXED
    from tandemproject_gb300.serve import Server
    from tandemproject_gb300.workloads import serving_requests
    out = {}
    for name, prec in (("mixed", MIXED), ("fp64", FP64)):
        reqs = serving_requests(args.serve_requests, seed=99, rate=4.0, step_scale=args.serve_step_scale,
                                precision=prec)
        done, summary = Server(budget_bytes=int(args.serve_budget_gb * 2 ** 30)).run(reqs)
        summary["workload"] = (f"{args.serve_requests} requests, seed 99, Poisson 4/s, 0.5-20 M points log-uniform, "
                               f"steps U[200,2000] x {args.serve_step_scale}, {args.serve_budget_gb:g} GB budget, "
                               f"{name}")
        summary["unit_latency"] = "s"
        out[name] = summary
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--preset", default="naca0012_8p8m")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--no-mixed", dest="mixed", action="store_false")
    ap.add_argument("--no-batch", dest="batch", action="store_false")
    ap.add_argument("--no-serve", dest="serve", action="store_false")
    ap.add_argument("--serve-requests", type=int, default=32)
    ap.add_argument("--serve-step-scale", type=float, default=0.1)
    ap.add_argument("--serve-budget-gb", type=float, default=40.0)
    ap.add_argument("--batch-steps", type=int, default=500)
    ap.add_argument("--batch-seq-steps", type=int, default=40)
    ap.add_argument("--mixed-preset", default="naca0012_25m")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    from tandemproject_gb300.config import PRESETS, FP64
    from tandemproject_gb300.grid import aerofoil_grid
    cfg = PRESETS[args.preset]
    ws, rank, local = dist_env()

    if args.impl == "reference":
        if rank != 0:
            return
        grid = aerofoil_grid(cfg)
        print(json.dumps(run_reference(args, cfg, grid)), flush=True)
        return

    import numpy as np
    import torch
    from tandemproject_gb300 import build as _b
    from tandemproject_gb300.solver import Case, probe_fma_tflops

    _b.build()
    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    grid = aerofoil_grid(cfg)
    case = Case(cfg)
    for mb in range(cfg.nblocks):
        case.set_grid(mb, grid[mb])
    case.init()
    npts = cfg.npoints
    stream = torch.cuda.ExternalStream(case.stream())

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    # warm-up (includes the dt = 0 start-up steps of the reference's schedule)
    case.step(args.warmup)
    barrier()
    l0 = case.launch_count()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        barrier()
        e0.record(stream)
        case.step(args.steps)
        e1.record(stream)
        barrier()
    ms = e0.elapsed_time(e1)
    launches = case.launch_count() - l0
    t_dev = ms / 1e3
    t_dev = max_over_ranks(t_dev, dist)
    value = npts * cfg.nkrk * args.steps * ws / t_dev

    # the mixed-precision path on the configuration it is quoted on (24.6 M points, 6 blocks 640 x 200 x 32), with
    # an FP64 run of the same case for the error and the FP64-vs-mixed speed-up on that case
    from tandemproject_gb300.config import MIXED
    mixed = None
    if args.mixed:
        mcfg = PRESETS[args.mixed_preset]
        mgrid = aerofoil_grid(mcfg)
        mn = mcfg.npoints
        runs = {}
        for name, prec in (("fp64", FP64), ("mixed", MIXED)):
            cm = Case(mcfg.replace(precision=prec))
            for mb in range(mcfg.nblocks):
                cm.set_grid(mb, mgrid[mb])
            cm.init()
            cm.step(args.warmup)
            barrier()
            sm = torch.cuda.ExternalStream(cm.stream())
            m0, m1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            m0.record(sm)
            cm.step(args.steps)
            m1.record(sm)
            barrier()
            t_run = m0.elapsed_time(m1) / 1e3
            t_run = max_over_ranks(t_run, dist)
            runs[name] = (cm, t_run)
        (cd, t_d), (cm, t_mix) = runs["fp64"], runs["mixed"]
        num = np.zeros(5)
        den = np.zeros(5)
        for mb in range(mcfg.nblocks):
            qd, qm = cd.get_state(mb), cm.get_state(mb)
            num += np.sum((qm - qd) ** 2, axis=1)
            den += np.sum(qd ** 2, axis=1)
        den[1:4] = den[1:4].sum()
        cd.close()
        cm.profile(True)
        cm.step(2)
        mprof = cm.profile_read()
        cm.profile(False)
        mtiles = cm.tiles()
        cm.close()
        mtot = sum(v[0] for v in mprof.values())
        mdom = max(mprof, key=lambda k: mprof[k][0])
        mkind = "filter" if mdom.startswith("filter") else "deriv"
        if mdom.startswith(("deriv", "filter")):
            munits = mn * FIELD_SWEEPS_PER_STEP[mkind] * 2 / max(mprof[mdom][1], 1)
            mt = mprof[mdom][0] / max(mprof[mdom][1], 1) / 1e3
            mach = SWEEP_BYTES_MIXED[mkind] * munits / mt / 1e9
            mroof = {"bound": "hbm", "kernel": f"k_sweep<{mdom}> in FP32, {SWEEP_BYTES_MIXED[mkind]} B per point-field",
                     "achieved": mach, "peak": measured_peaks()[0], "unit": "GB/s",
                     "frac": mach / measured_peaks()[0]}
        elif mdom in POINTWISE_BYTES_MIXED and mcfg.nviscous == 1:
            mt = mprof[mdom][0] / max(mprof[mdom][1], 1) / 1e3
            mach = POINTWISE_BYTES_MIXED[mdom] * mn / mt / 1e9
            mroof = {"bound": "hbm", "kernel": "k_flux_staged (viscous fluxes, stresses at the point), "
                                               f"{POINTWISE_BYTES_MIXED[mdom]} B per point",
                     "achieved": mach, "peak": measured_peaks()[0], "unit": "GB/s",
                     "frac": mach / measured_peaks()[0]}
        else:
            mroof = {"kernel": mdom, "note": "no algorithmic byte count for this kernel class"}
        v_mix = mn * mcfg.nkrk * args.steps * ws / t_mix
        v_d = mn * mcfg.nkrk * args.steps * ws / t_d
        mixed = {"workload": f"{args.mixed_preset}: NACA 0012, 6 blocks "
                             f"{'x'.join(str(v + 1) for v in (mcfg.lxibk[0], mcfg.letbk[0], mcfg.lzebk[0]))}, "
                             f"{mn} points, impulsive start, {args.steps} steps after {args.warmup} warm-up",
                 "value": v_mix, "ms_per_step": t_mix / args.steps * 1e3,
                 "fp64_same_case": {"value": v_d, "ms_per_step": t_d / args.steps * 1e3},
                 "dtype": "f32 line solves/filters/fluxes, f64 metrics, Jacobian and RK state",
                 "speedup_vs_fp64": v_mix / v_d,
                 "rel_l2_vs_fp64_after_steps": {"steps": args.warmup + args.steps,
                                                "rho": float(np.sqrt(num[0] / den[0])),
                                                "momentum": float(np.sqrt(num[1:4].sum() / den[1])),
                                                "rhoE": float(np.sqrt(num[4] / den[4]))},
                 "stage_hbm_frac_728B": STAGE_BYTES_MIXED * (mn * mcfg.nkrk * args.steps / t_mix) / 1e9
                 / measured_peaks()[0],
                 "roofline": mroof,
                 "tiles": list(mtiles),
                 "kernel_share": {k: round(v[0] / mtot, 4) for k, v in mprof.items() if v[1]}}

    # end to end through the C ABI: pinned host state in (one copy of every block), step, state out
    host = torch.empty(5 * case.points_total(), dtype=torch.float64, pin_memory=True)
    hnp = host.numpy()
    case.get_state_all(out=hnp)
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        case.set_state_all(hnp)
        case.step(1)
        case.get_state_all(out=hnp)
    barrier()
    t_e2e = time.perf_counter() - t0
    t_e2e = max_over_ranks(t_e2e, dist)
    bytes_state = 5 * npts * 8
    e2e = {"value": npts * cfg.nkrk * args.e2e_steps * ws / t_e2e, "unit": UNIT,
           "h2d_bytes_per_step": bytes_state, "d2h_bytes_per_step": bytes_state, "steps": args.e2e_steps}

    # roofline of the dominant kernel class from profiled launches
    case.profile(True)
    case.step(2)
    prof = case.profile_read()
    case.profile(False)
    tot = sum(v[0] for v in prof.values())
    dom = max(prof, key=lambda k: prof[k][0])
    hbm_peak, peak_src = measured_peaks()
    fp64_peak = probe_fma_tflops(True)

    def sweep_roofline(cls):
        """roofline of one line-sweep class: units (point x field) one launch processes, on average over the
        profiled steps, at that class's average launch duration"""
        ms, n = prof[cls]
        kind = "filter" if cls.startswith("filter") else "deriv"
        units = npts * FIELD_SWEEPS_PER_STEP[kind] * 2 / max(n, 1)
        t = ms / max(n, 1) / 1e3
        ach = SWEEP_BYTES[kind] * units / t / 1e9
        ach64 = SWEEP_FLOPS[kind] * units / t / 1e12
        return {"bound": "hbm", "achieved": ach, "peak": hbm_peak, "unit": "GB/s", "frac": ach / hbm_peak,
                "traffic": SWEEP_TRAFFIC_PER_UNIT[cls] * units if cls in SWEEP_TRAFFIC_PER_UNIT else None,
                "traffic_source": "ncu DRAM bytes per unit of one launch on the 3.54 M-point case, scaled by units",
                "kernel": f"k_sweep<{cls}>: one launch = every line of one direction over all blocks for "
                          f"{units / npts:.1f} fields on average ({units:.3e} point-fields), "
                          f"{SWEEP_BYTES[kind]} B and {SWEEP_FLOPS[kind]} flop per point-field",
                "fp64": {"achieved_tflops": ach64, "peak_tflops": fp64_peak, "frac": ach64 / fp64_peak}}

    sweep_cls = max((k for k in prof if k.startswith(("deriv", "filter")) and prof[k][1]), key=lambda k: prof[k][0])
    if dom == "flux" and cfg.nviscous == 1:
        # the viscous flux kernel with the stresses at the point (k_flux_visc): one launch covers every point
        ms, n = prof["flux"]
        t = ms / max(n, 1) / 1e3
        achieved = FLUX_BYTES_FP64 * npts / t / 1e9
        fp64_ach = FLUX_FLOPS_FP64 * npts / t / 1e12
        roofline = {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                    "frac": achieved / hbm_peak,
                    "traffic": FLUX_TRAFFIC_PER_POINT * npts if FLUX_TRAFFIC_PER_POINT else None,
                    "traffic_source": "ncu DRAM bytes per point of one launch on the 3.54 M-point case, scaled by "
                                      "points",
                    "kernel": f"k_flux_visc (viscous fluxes with the stresses at the point): one launch = every point "
                              f"({npts}), {FLUX_BYTES_FP64} B and {FLUX_FLOPS_FP64} FP64 flop per point",
                    "fp64": {"achieved_tflops": fp64_ach, "peak_tflops": fp64_peak, "frac": fp64_ach / fp64_peak}}
    elif dom.startswith(("deriv", "filter")):
        roofline = sweep_roofline(dom)
    else:  # (a class with no algorithmic count leads only when launches are serialised, e.g. under a profiler)
        roofline = sweep_roofline(sweep_cls)
        roofline["note"] = f"largest class {dom} has no algorithmic byte count; the largest sweep class is shown"
    roofline["fp64"]["peak_source"] = "measured FP64 FMA throughput of this GPU (ati_probe_fma_tflops)"
    roofline.update({
        "peak_source": f"{peak_src} (MEASURED_PEAKS.json hbm_gbs)",
        "limit": "the FP64 pipe (ncu: 89-92 % busy in the line sweeps and the flux kernel at 12-34 % of HBM); "
                 "frac is against HBM, fp64.frac against the FP64 FMA peak",
        "stage_hbm_frac": STAGE_BYTES_FP64 * value / ws / 1e9 / hbm_peak,
        "kernel_share": {k: round(v[0] / tot, 4) for k, v in prof.items() if v[1]}})
    if dom != sweep_cls and "note" not in roofline:
        roofline["largest_sweep"] = sweep_roofline(sweep_cls)

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_dev / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic: NACA 0012 grid from the reference's grid generator (restated), uniform freestream "
                    "initial state, " + ("impulsive start (nsmf = 1)" if cfg.nsmf == 1 else
                                         f"the reference deck's smooth start (nsmf = 0, timf = {cfg.timf:g})") +
                    "; seeded von Karman inflow turbulence when the preset has it (2.5 % of U_inf, L = 0.1 c, "
                    "2048 modes, seed 1234)",
            "config": {"workload": f"{args.preset}: NACA 0012, 6 blocks "
                                   f"{'x'.join(str(v + 1) for v in (cfg.lxibk[0], cfg.letbk[0], cfg.lzebk[0]))}, "
                                   f"{npts} points, FP64, RK4, Re 4e5, M 0.24",
                       "points": npts, "parallelism": f"replicas x{ws}" if ws > 1 else "single GPU",
                       "l2": "no flush: the state alone (5 x 8 B x points) exceeds the 129 MB L2",
                       "tiles": dict(zip(("xi_lines_per_cta", "eta_lines_per_cta", "zeta_lines_per_cta",
                                          "points_per_tile"),
                                         case.tiles()))},
            "e2e": e2e, "roofline": roofline, "clocks": clk.summary(), "gpu_launches": launches}
    if mixed is not None:
        line["mixed"] = mixed
    case.close()
    if args.batch:
        line["batch"] = batch_leg(args, barrier)
    if args.serve and rank == 0:
        line["serving"] = serve_leg(args)
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(cfg, grid)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
