"""FP32-residual accuracy against the FP64 path, at each benchmark configuration's own horizon.

    python -m opensbli_gb300.accuracy --size 256 --steps 1000 --every 50 --out result.json
    python -m opensbli_gb300.accuracy --workload tgv64 --steps 500 --every 50
    python -m opensbli_gb300.accuracy --workload kh_ensemble --steps 2000 --every 200
    python -m opensbli_gb300.accuracy --workload curv4 --steps 500 --every 50
    python -m opensbli_gb300.accuracy --workload channel --steps 500 --every 50
    python -m opensbli_gb300.accuracy --workload tcf --steps 500 --every 50

Advances, in lockstep from the same initial state, the FP64 path (the reference solution),
the FP32-residual path (FP64 state, RK register and reductions) and -- with --floor -- a second
FP64 run whose initial state carries a relative perturbation of `floor_amp` (seeded), for
`steps` RK3 steps.  Every `every` steps it records the relative L2 / Linf differences of rho and
rhoE against the FP64 run (L2 over the interior points of every block; Linf = max |diff| over
max |field|) and the kinetic energy of every run.  The perturbed FP64 run measures how fast the
flow amplifies any difference at rounding level: the floor that no implementation differing
from the FP64 path by rounding can stay under.

Workloads: tgv (the supersonic TGV at --size^3, CFL 0.5 at t = 0, --scheme), tgv64 (the 64^3
low-Mach TGV with the central scheme, dt 3.385e-3), kh_ensemble (the 64 seeded Kelvin-Helmholtz
instances, dt 2e-4, the FP32 run on the persistent batched stage), curv4 (the 4-block 3D
curvilinear case, CFL 0.5 at t = 0), channel (the 256 x 257 x 128 channel between isothermal
walls, dt 2e-4), tcf (the TENO turbulent-channel app's discretisation at its 129^3, SSP RK3,
dt 2e-4).
"""
import argparse
import json
import time

import numpy as np

from . import abi, problems
from .solver import Solver


def _diff(torch, runs_a, runs_b, specs):
    """rel L2 / Linf of rho and rhoE of run a against run b over all blocks."""
    out = {}
    for name in ("rho", "rhoE"):
        num = den = 0.0
        dmax = fmax = 0.0
        for ib, spec in enumerate(specs):
            v = 0 if name == "rho" else spec.nvars - 1
            sl = spec.interior()
            x = runs_a[ib][v][sl]
            y = runs_b[ib][v][sl]
            d = x - y
            num += float(torch.sum(d * d))
            den += float(torch.sum(y * y))
            dmax = max(dmax, float(d.abs().max()))
            fmax = max(fmax, float(y.abs().max()))
        out[name] = {"rel_l2": (num / den) ** 0.5, "rel_linf": dmax / fmax}
    return out


def workload(name, size=256, scheme=abi.SCHEME_TENO5, averaging=abi.AVG_ROE, minf=1.25, cfl=0.5):
    """(blocks, dt, rk, description) of a benchmark configuration."""
    if name == "tgv":
        spec, q = problems.tgv(size, minf=minf, scheme=scheme, averaging=averaging)
        return [(spec, q)], problems.cfl_dt(spec, q, cfl), "ls3", "supersonic TGV %d^3 (CFL %.1f)" % (size, cfl)
    if name == "tgv64":
        return ([problems.tgv(64, minf=0.1, scheme=abi.SCHEME_CENTRAL4)], 3.385e-3, "ls3",
                "TGV 64^3, M=0.1, central-4 Feiereisen + viscous, dt 3.385e-3")
    if name == "kh_ensemble":
        return (problems.kh_ensemble(64, seed=0), 2e-4, "ls3",
                "64 Kelvin-Helmholtz instances (seed 0), WENO5-Z (Roe), dt 2e-4")
    if name == "curv4":
        blocks = problems.curvilinear_multiblock_3d(seed=0)
        return blocks, problems.multiblock_cfl_dt(blocks, cfl), "ls3", "4-block 3D curvilinear TENO5 (CFL 0.5)"
    if name == "channel":
        return ([problems.channel_iso((256, 257, 128))], 2e-4, "ls3",
                "channel 256 x 257 x 128 between isothermal walls, TENO5 + viscous (Carpenter closures), dt 2e-4")
    if name == "tcf":
        return ([problems.channel_tcf((129, 129, 129))], 2e-4, (abi.RK_LOW_STORAGE, problems.RK3_SSP_A,
                                                               problems.RK3_SSP_B),
                "the TENO turbulent-channel app's discretisation at 129^3 (TENO6, mu = T^0.7, forcing, "
                "stretched walls, SSP RK3), dt 2e-4")
    raise ValueError("unknown workload %s" % name)


def run(size=256, steps=1000, every=50, scheme=abi.SCHEME_TENO5, averaging=abi.AVG_ROE, minf=1.25, cfl=0.5,
        floor=False, floor_amp=1e-12, seed=0, fp32=True, name="tgv"):
    blocks, dt, rk, desc = workload(name, size, scheme, averaging, minf, cfl)
    specs = [b[0] for b in blocks]
    runs = {"fp64": Solver(blocks, precision="fp64", rk=rk)}
    if fp32:
        runs["fp32"] = Solver(blocks, precision="fp32", rk=rk)
    if floor:
        rng = np.random.default_rng(seed)
        pert = [(b[0], [a * (1.0 + floor_amp * rng.standard_normal(a.shape)) for a in b[1]]) + tuple(b[2:])
                for b in blocks]
        runs["fp64_perturbed"] = Solver(pert, precision="fp64", rk=rk)
    torch = runs["fp64"].torch
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
        for k in hist["diff"]:
            hist["diff"][k].append(_diff(torch, runs[k].q, runs["fp64"].q, specs))
    npts = sum(s.npoints for s in specs)
    out = {"workload": name, "description": desc, "points": npts, "size": size, "steps": steps, "dt": dt,
           "scheme": scheme, "averaging": averaging, "minf": minf,
           "floor_amp": floor_amp if floor else None, "history": hist, "seconds": secs,
           "mpt_stage_per_s": {k: npts * 3 * steps / secs[k] / 1e6 for k in secs}}
    out["errors"] = {k: v[-1] for k, v in hist["diff"].items()}
    ke64 = np.array(hist["ke"]["fp64"])
    out["ke_max_rel_dev"] = {k: float(np.max(np.abs(np.array(v) - ke64) / np.abs(ke64)))
                             for k, v in hist["ke"].items() if k != "fp64"}
    for s in runs.values():
        s.close()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="tgv", choices=["tgv", "tgv64", "kh_ensemble", "curv4", "channel", "tcf"])
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
              floor_amp=args.floor_amp, fp32=not args.no_fp32, name=args.workload)
    txt = json.dumps(res)
    print(json.dumps({"workload": args.workload, "errors": res["errors"], "ke_max_rel_dev": res["ke_max_rel_dev"],
                      "mpt_stage_per_s": res["mpt_stage_per_s"]}))
    if args.out:
        with open(args.out, "w") as f:
            f.write(txt + "\n")


if __name__ == "__main__":
    main()
