"""Run one of the benchmark configurations for a number of steps on the GPU (for profiling and
quick checks; the throughput measurement with its roofline and baselines is bench.py).

    python -m opensbli_gb300.run tgv --size 160 --precision fp32 --steps 1
    python -m opensbli_gb300.run curv4 --xy-scale 2 --precision fp32 --steps 1
    python -m opensbli_gb300.run kh --count 16 --steps 1
    python -m opensbli_gb300.run sod --precision fp64 --steps 50
    python -m opensbli_gb300.run tgv --size 160 --central-staging 1 --steps 1
    python -m opensbli_gb300.run channel --size 128 --steps 1

tgv: the supersonic TGV (TENO5, Roe average, central viscous terms) at --size^3, dt 1e-3;
curv4: the 4-block curvilinear case with its x and y sizes divided by --xy-scale;
kh: the first --count instances of the seeded KH ensemble on the persistent stage;
sod: the 400-point Sod tube (one osb_step call, the resident path);
channel: the channel between isothermal walls (TENO5 + viscous, Carpenter closures) of
--size x (--size + 1) x --size/2 points, dt 2e-4.
Graphs are off and the FP32 per-block path applies the RK update in its last kernel, whose
central kernel stages its planes by register loads (--central-staging 0, the default) or bulk
copies (1).
"""
import argparse
import sys

from . import abi, problems
from .solver import Solver


def build(args):
    if args.workload == "tgv":
        spec, q = problems.tgv(args.size, minf=1.25, scheme=abi.SCHEME_TENO5, averaging=abi.AVG_ROE)
        return [(spec, q)], 1e-3, {"mode": abi.SCHED_PER_BLOCK, "fuse_update": 1}
    if args.workload == "curv4":
        sizes = {k: (s[0] // args.xy_scale, s[1] // args.xy_scale, s[2]) for k, s in problems.MB_SIZES.items()}
        blocks = problems.curvilinear_multiblock_3d(sizes=sizes, seed=0)
        return blocks, problems.multiblock_cfl_dt(blocks, 0.5), {"mode": abi.SCHED_PER_BLOCK}
    if args.workload == "kh":
        return (problems.kh_ensemble(args.count, seed=0), 2e-4,
                {"mode": abi.SCHED_PERSISTENT, "tile_y": 16, "ctas_per_sm": 2, "dynamic": 1, "order": 0})
    if args.workload == "sod":
        return [problems.sod(400)], 2e-4, None
    if args.workload == "channel":
        n = args.size
        return [problems.channel_iso((n, n + 1, n // 2))], 2e-4, {"mode": abi.SCHED_PER_BLOCK, "fuse_update": 1}
    raise ValueError(args.workload)


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("workload", choices=["tgv", "curv4", "kh", "sod", "channel"])
    ap.add_argument("--size", type=int, default=160)
    ap.add_argument("--xy-scale", type=int, default=1)
    ap.add_argument("--count", type=int, default=16)
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64"])
    ap.add_argument("--steps", type=int, default=1)
    ap.add_argument("--central-staging", type=int, default=0, choices=[0, 1])
    args = ap.parse_args(argv)
    blocks, dt, sched = build(args)
    precision = "fp32" if args.workload == "kh" else args.precision
    s = Solver(blocks, precision=precision, rk="ls3", graphs=False)
    if sched is not None:
        s.set_schedule(**sched)
    s.set_central_staging(args.central_staging)
    s.apply_bc()
    s.step(dt, args.steps)
    s.sync()
    print("ok: %d points, %d launches" % (sum(b[0].npoints for b in blocks), s.launches()))
    s.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
