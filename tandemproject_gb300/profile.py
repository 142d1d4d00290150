"""Per-kernel-class timings of the fused time step, through the library's own
profiling calls (ati_profile_enable / ati_profile_read: CUDA events around
every launch on the case's stream).

The case first steps `--warmup` times through its CUDA graph, then `--steps`
times through the graph (wall clock around the steps: the graph-timed step),
then `--steps` times with the events; the table gives per class the time per
launch, the launches and the share of the profiled time.  `--fused` switches
the fused face chains on, `--no-tma` and `--no-pairs` the TMA staging and the
paired-line sweeps off, `--dense-zeta` the dense zeta derivatives on (ati_set_options).

    python -m tandemproject_gb300.profile [--preset NAME] [--precision fp64|mixed|strict]
                                          [--steps K] [--warmup W] [--fused] [--no-tma] [--no-pairs] [--dense-zeta]
                                          [--json]
"""
import argparse
import json
import sys
import time


def profile_case(preset="naca0012_8p8m", precision="fp64", steps=10, warmup=3, fused=False, tma=True, pairs=True,
                 timing=None, dense_zeta=False):
    """{class: (microseconds per launch, launches, share)}, tiles, ms per step.  `timing` (a dict) receives the
    graph-timed milliseconds per step and the options in effect."""
    from .config import FP64, FP64_STRICT, MIXED, PRESETS
    from .solver import setup_case
    prec = {"fp64": FP64, "mixed": MIXED, "strict": FP64_STRICT}[precision]
    case = setup_case(PRESETS[preset].replace(precision=prec))
    try:
        opts = case.set_options(tma=tma, fused_faces=fused, paired_lines=pairs, dense_zeta=dense_zeta)
        case.step(warmup)
        case.synchronize()
        t0 = time.perf_counter()
        case.step(steps)
        case.synchronize()
        if timing is not None:
            timing["graph_ms_per_step"] = 1000.0 * (time.perf_counter() - t0) / steps
            timing["options"] = opts
        case.profile(True)
        case.step(steps)
        prof = case.profile_read()
        case.profile(False)
        tiles = list(case.tiles())
    finally:
        case.close()
    total = sum(ms for ms, _ in prof.values())
    rows = {k: (1000.0 * ms / n, n, ms / total) for k, (ms, n) in prof.items() if n}
    return rows, tiles, total / steps


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--preset", default="naca0012_8p8m")
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed", "strict"])
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--fused", action="store_true")
    ap.add_argument("--no-tma", action="store_true")
    ap.add_argument("--no-pairs", action="store_true")
    ap.add_argument("--dense-zeta", action="store_true")
    ap.add_argument("--json", action="store_true")
    a = ap.parse_args(argv)
    tm = {}
    rows, tiles, ms_step = profile_case(a.preset, a.precision, a.steps, a.warmup, a.fused, not a.no_tma,
                                        not a.no_pairs, tm, a.dense_zeta)
    if a.json:
        print(json.dumps({"preset": a.preset, "precision": a.precision, "tiles": tiles, "ms_per_step": ms_step,
                          "graph_ms_per_step": tm["graph_ms_per_step"], "options": tm["options"],
                          "classes": {k: {"us_per_launch": v[0], "launches": v[1], "share": v[2]}
                                      for k, v in rows.items()}}))
        return 0
    print(f"{a.preset} {a.precision}: tiles {tiles}, options {tm['options']}, "
          f"{tm['graph_ms_per_step']:.3f} ms per graph step, {ms_step:.3f} ms per profiled step")
    for k, (us, n, share) in rows.items():
        print(f"  {k:<14s} {us:9.1f} us/launch {n:6d} launches {100 * share:6.1f} %")
    return 0


if __name__ == "__main__":
    sys.exit(main())
