"""FP32-residual accuracy against the FP64 path on the supersonic Taylor-Green vortex.

    python -m opensbli_gb300.accuracy --size 256 --steps 1000 --every 50 --out result.json

Runs the same initial state with the FP64 path and with the FP32-residual path (FP64 state,
RK register and reductions) for `steps` RK3 steps at the CFL-0.5 time step of t=0, records the
kinetic-energy history of both every `every` steps and reports the relative L2 / Linf errors
of rho and rhoE at the end, and the largest relative KE-history deviation.
"""
import argparse
import json
import time

import numpy as np

from . import abi, problems
from .solver import Solver


def run(size=256, steps=1000, every=50, scheme=abi.SCHEME_TENO5, averaging=abi.AVG_ROE, minf=1.25, cfl=0.5):
    spec, q = problems.tgv(size, minf=minf, scheme=scheme, averaging=averaging)
    dt = problems.cfl_dt(spec, q, cfl)
    out = {"size": size, "steps": steps, "dt": dt, "scheme": scheme, "averaging": averaging, "minf": minf}
    states, hist, secs = {}, {}, {}
    for prec in ("fp32", "fp64"):
        s = Solver([(spec, q)], precision=prec, rk="ls3")
        s.apply_bc()
        h = [(0, s.reduce(abi.RED_KE))]
        t0 = time.time()
        done = 0
        while done < steps:
            n = min(every, steps - done)
            s.step(dt, n)
            done += n
            s.sync()
            h.append((done, s.reduce(abi.RED_KE)))
        secs[prec] = time.time() - t0
        states[prec] = s.state(0)
        hist[prec] = h
        s.close()
    sl = spec.interior()
    errs = {}
    for v, name in ((0, "rho"), (spec.nvars - 1, "rhoE")):
        a, b = states["fp32"][v][sl], states["fp64"][v][sl]
        d = a - b
        errs[name] = {"rel_l2": float(np.linalg.norm(d) / np.linalg.norm(b)),
                      "rel_linf": float(np.max(np.abs(d)) / np.max(np.abs(b)))}
    ke32 = np.array([k for _, k in hist["fp32"]])
    ke64 = np.array([k for _, k in hist["fp64"]])
    out["errors"] = errs
    out["ke_history"] = {"steps": [n for n, _ in hist["fp64"]], "fp64": ke64.tolist(), "fp32": ke32.tolist(),
                         "max_rel_dev": float(np.max(np.abs(ke32 - ke64) / np.abs(ke64)))}
    out["seconds"] = secs
    out["mpt_stage_per_s"] = {p: spec.npoints * 3 * steps / secs[p] / 1e6 for p in secs}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--size", type=int, default=256)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--every", type=int, default=50)
    ap.add_argument("--scheme", default="teno5", choices=sorted(abi.SCHEME_NAMES))
    ap.add_argument("--out", default=None)
    args = ap.parse_args()
    scheme = abi.SCHEME_NAMES[args.scheme]
    avg = abi.AVG_ROE if scheme == abi.SCHEME_TENO5 else abi.AVG_SIMPLE
    res = run(args.size, args.steps, args.every, scheme=scheme, averaging=avg)
    txt = json.dumps(res)
    print(txt)
    if args.out:
        with open(args.out, "w") as f:
            f.write(txt + "\n")


if __name__ == "__main__":
    main()
