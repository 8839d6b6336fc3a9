"""FP32-residual accuracy against the FP64 path on the supersonic Taylor-Green vortex.

    python -m opensbli_gb300.accuracy --size 256 --steps 1000 --every 50 --out result.json

Advances, in lockstep from the same initial state, the FP64 path (the reference solution),
the FP32-residual path (FP64 state, RK register and reductions) and -- with --floor -- a second
FP64 run whose initial state carries a relative perturbation of `floor_amp` (seeded), for
`steps` RK3 steps at the CFL-0.5 time step of t = 0.  Every `every` steps it records the
relative L2 / Linf differences of rho and rhoE against the FP64 run and the kinetic energy of
every run.  The perturbed FP64 run measures how fast this flow amplifies any difference at
rounding level: it is the floor that no implementation differing from the FP64 path by
rounding can stay under.
"""
import argparse
import json
import time

import numpy as np

from . import abi, problems
from .solver import Solver


def _diff(torch, a, b, sl):
    out = {}
    for v, name in ((0, "rho"), (a.shape[0] - 1, "rhoE")):
        x = a[v][sl]
        y = b[v][sl]
        d = x - y
        out[name] = {"rel_l2": float(torch.linalg.vector_norm(d) / torch.linalg.vector_norm(y)),
                     "rel_linf": float(d.abs().max() / y.abs().max())}
    return out


def run(size=256, steps=1000, every=50, scheme=abi.SCHEME_TENO5, averaging=abi.AVG_ROE, minf=1.25, cfl=0.5,
        floor=False, floor_amp=1e-12, seed=0, fp32=True):
    spec, q = problems.tgv(size, minf=minf, scheme=scheme, averaging=averaging)
    dt = problems.cfl_dt(spec, q, cfl)
    runs = {"fp64": Solver([(spec, q)], precision="fp64", rk="ls3")}
    if fp32:
        runs["fp32"] = Solver([(spec, q)], precision="fp32", rk="ls3")
    if floor:
        rng = np.random.default_rng(seed)
        qp = [a * (1.0 + floor_amp * rng.standard_normal(a.shape)) for a in q]
        runs["fp64_perturbed"] = Solver([(spec, qp)], precision="fp64", rk="ls3")
    torch = runs["fp64"].torch
    h = spec.halo
    sl = tuple(slice(h, h + spec.size[d]) for d in reversed(range(spec.ndim)))
    for s in runs.values():
        s.apply_bc()
    hist = {"steps": [0], "ke": {k: [s.reduce(abi.RED_KE)] for k, s in runs.items()},
            "diff": {k: [] for k in runs if k != "fp64"}}
    secs = {k: 0.0 for k in runs}
    done = 0
    while done < steps:
        n = min(every, steps - done)
        for k, s in runs.items():
            t0 = time.time()
            s.step(dt, n)
            s.sync()
            secs[k] += time.time() - t0
        done += n
        hist["steps"].append(done)
        for k, s in runs.items():
            hist["ke"][k].append(s.reduce(abi.RED_KE))
        ref = runs["fp64"].q[0]
        for k in hist["diff"]:
            hist["diff"][k].append(_diff(torch, runs[k].q[0], ref, sl))
    out = {"size": size, "steps": steps, "dt": dt, "scheme": scheme, "averaging": averaging, "minf": minf,
           "floor_amp": floor_amp if floor else None, "history": hist, "seconds": secs,
           "mpt_stage_per_s": {k: spec.npoints * 3 * steps / secs[k] / 1e6 for k in secs}}
    out["errors"] = {k: v[-1] for k, v in hist["diff"].items()}
    ke64 = np.array(hist["ke"]["fp64"])
    out["ke_max_rel_dev"] = {k: float(np.max(np.abs(np.array(v) - ke64) / np.abs(ke64)))
                             for k, v in hist["ke"].items() if k != "fp64"}
    for s in runs.values():
        s.close()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--size", type=int, default=256)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--every", type=int, default=50)
    ap.add_argument("--scheme", default="teno5", choices=sorted(abi.SCHEME_NAMES))
    ap.add_argument("--floor", action="store_true", help="also run the perturbed FP64 sensitivity floor")
    ap.add_argument("--floor-amp", type=float, default=1e-12)
    ap.add_argument("--no-fp32", action="store_true", help="only the FP64 run and its perturbed twin")
    ap.add_argument("--out", default=None)
    args = ap.parse_args()
    scheme = abi.SCHEME_NAMES[args.scheme]
    avg = abi.AVG_ROE if scheme == abi.SCHEME_TENO5 else abi.AVG_SIMPLE
    res = run(args.size, args.steps, args.every, scheme=scheme, averaging=avg, floor=args.floor,
              floor_amp=args.floor_amp, fp32=not args.no_fp32)
    txt = json.dumps(res)
    print(json.dumps({"errors": res["errors"], "ke_max_rel_dev": res["ke_max_rel_dev"],
                      "mpt_stage_per_s": res["mpt_stage_per_s"]}))
    if args.out:
        with open(args.out, "w") as f:
            f.write(txt + "\n")


if __name__ == "__main__":
    main()
