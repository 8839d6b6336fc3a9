"""Benchmark: Mpt-RK-stage updates/s of the explicit residual + RK3 path on the 256^3
supersonic Taylor-Green vortex (M=1.25, Re=1600, TENO5 with Roe averaging + 4th-order central
viscous terms, periodic, low-storage RK3, dt from CFL 0.5 at t=0), FP32 residual with FP64
state, next to the plain FP64 path, the reference's OPS solver on the host cores, and the
kernel roofline.

    python bench.py [--gpus 1] [--steps K] [--warmup W] [--impl reference]

One "step" is one full RK step (3 stages) of the whole 256^3 block.  The state (5 x 266^3
FP64, 752 MB) is larger than L2 (129 MB), so no explicit L2 flush is needed between steps.
Replicas only for N > 1 (independent blocks per rank, no collective on the data path).
"""
import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import faulthandler

import numpy as np

faulthandler.enable()
ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mpt-RK-stage updates/s (FP32 residual, FP64 state)"
UNIT = "Mpt-RK-stage/s"
NS = 256
MINF = 1.25
CFL = 0.5
BYTES_PER_PT_STAGE = 160.0  # fully fused algorithmic traffic: q and RKold read+written once, FP64
# FP32-residual vs FP64 after the configuration's own 1000 steps (256^3, CFL 0.5), measured by
# `python -m opensbli_gb300.accuracy --size 256 --steps 1000` (profiles/accuracy_tgv256_fp32_vs_fp64.md);
# too long (about 9 minutes of FP64 steps) to repeat inside the bench
ACCURACY_1000 = {
    "source": "profiles/accuracy_tgv256_fp32_vs_fp64.md (python -m opensbli_gb300.accuracy --size 256 --steps 1000)",
    "teno5_roe": {"rho": {"rel_l2": 1.13e-4, "rel_linf": 1.03e-2}, "rhoE": {"rel_l2": 1.39e-4, "rel_linf": 6.90e-3},
                  "ke_max_rel_dev": 1.57e-6,
                  "fp64_with_1e-8_input_perturbation": {"rho_rel_l2": 1.10e-4, "rhoE_rel_l2": 1.33e-4}},
    "weno5z_simple": {"rho": {"rel_l2": 1.75e-7, "rel_linf": 9.83e-6},
                      "rhoE": {"rel_l2": 2.16e-7, "rel_linf": 1.43e-5}, "ke_max_rel_dev": 5.26e-8},
    "note": "weno5z_simple measured with the difference-form central derivatives; teno5_roe with the "
            "earlier weighted-sum form (its 1000-step error is the TENO5 cut-off's amplification of any "
            "1e-8 difference, the same as the FP64 run's with a 1e-8 input perturbation)",
    "target_rel_l2": 1e-5,
    "target_met": {"teno5_roe": False, "weno5z_simple": True},
}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--size", type=int, default=NS)
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--workload", default="tgv",
                    choices=["tgv", "sod", "tgv64", "kh_ensemble", "curv4", "c4w5", "tvd", "shock", "channel", "tcf"],
                    help="tgv: the 256^3 supersonic TGV (headline); sod: the 400-point Sod tube; tgv64: the "
                         "64^3 central TGV; kh_ensemble: 64 uneven 2D Kelvin-Helmholtz instances in one "
                         "persistent launch per stage; curv4: the 4-block 3D curvilinear TENO5 case; c4w5: the "
                         "Central4-WENO5 benchmark's TGV (central KGP + WENO filter) at --size^3; tvd: the TGV "
                         "app's TVD branch (central KGP + TVD filter) at --size^3; shock: the 2D inviscid shock "
                         "reflection app (457 x 255, Dirichlet / extrapolation / symmetry boundaries); channel: a "
                         "3D channel between isothermal no-slip walls (TENO5 + viscous terms with the Carpenter "
                         "closures), 256 x 257 x 128; tcf: the TENO turbulent-channel app's discretisation at its "
                         "129^3 (TENO6, power-law viscosity, forcing, stretched walls, SSP RK3)")
    ap.add_argument("--ensemble", type=int, default=64)
    ap.add_argument("--variant", type=int, default=0, help="x-sweep tiling variant when --fuse is given")
    ap.add_argument("--fuse", default="auto", choices=["auto", "0", "1"],
                    help="RK update inside the central kernel (1), as its own kernel (0), or the fastest "
                         "schedule (fusion and x-sweep tiling) as timed by the autotuner (auto)")
    ap.add_argument("--no-tune", action="store_true")
    return ap.parse_args()


def dist_env():
    from opensbli_gb300.replicas import dist_env as env
    return env()


class ClockSampler:
    """Samples nvidia-smi SM clocks and throttle reasons while the timed region runs."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.QUERY,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def stop(self):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        if self.thread is not None:
            self.thread.join(timeout=2)
        return self.summary()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for i, n in enumerate(names):
                if r[5 + i].lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


def measured_traffic(kernel, fused):
    """DRAM bytes (read + write) per point of one launch of `kernel`, from the ncu capture
    summarised in profiles/dram_traffic_tgv_fp32.txt (captured on the 256^3 block; traffic
    scales with the points of the block), or None."""
    path = os.path.join(ROOT, "profiles", "dram_traffic_tgv_fp32.txt")
    if not os.path.exists(path):
        return None
    key = kernel + ("_fused" if kernel == "central" and fused else "")
    for line in open(path):
        parts = line.split("#")[0].split()
        if len(parts) >= 2 and parts[0] == key:
            return float(parts[1])
    return None


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


def probe_fp(device):
    import ctypes
    path = os.path.join(ROOT, "opensbli_gb300", "libosb_probe.so")
    if not os.path.exists(path):
        return None, None
    lib = ctypes.CDLL(path)
    lib.osb_probe_fma.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
    out = {}
    for name, fp64 in (("fp32", 0), ("fp64", 1)):
        v = ctypes.c_double()
        rc = lib.osb_probe_fma(device, fp64, ctypes.byref(v))
        out[name] = v.value / 1e12 if rc == 0 else None
    return out["fp32"], out["fp64"]


def log(msg):
    sys.stderr.write("[bench] %s\n" % msg)
    sys.stderr.flush()


def make_problem(n):
    from opensbli_gb300 import abi, problems
    spec, q = problems.tgv(n, minf=MINF, scheme=abi.SCHEME_TENO5, averaging=abi.AVG_ROE)
    dt = problems.cfl_dt(spec, q, CFL)
    return spec, q, dt


def kernel_bytes(fused, nv=5, ndim=3, curvilinear=False, a_zero_stages=1, nstages=3, central_only=False):
    """Algorithmic bytes per point of one launch of each FP32-path kernel, averaged over the
    stages of a step: its own minimal inputs and outputs (FP32 state nv x 4 B, float-float
    residual nv x 8 B, FP64 state and RK register nv x 8 B each; a curvilinear sweep also reads
    its metric row and det J in FP32, (ndim + 1) x 4 B).  The first low-storage stage (A = 0)
    does not read the register: a_zero_stages of the nstages read nv x 8 B less.  central_only:
    the central kernel is the block's only residual kernel (central scheme), so it reads no
    partial residual."""
    st = 4.0 * nv
    res = 8.0 * nv
    met = 4.0 * (ndim + 1) if curvilinear else 0.0
    reg_read = 8.0 * nv * (nstages - a_zero_stages) / nstages
    upd = 8.0 * nv + reg_read + 16.0 * nv + st  # state read, register read, both written, FP32 out
    return {"flux_x": st + met + res,              # read FP32 state, write residual
            "flux_y": st + met + 2 * res,          # read FP32 state, read + write residual
            "flux_z": st + met + 2 * res,
            "central": (st + (0.0 if central_only else res) + upd) if fused else
                       (st + (res if central_only else 2 * res)),
            "rk_update": res + upd,                # residual in, the update's arrays
            "boundary": 0.0, "reduce": 8.0 * nv, "persistent_stage": 0.0}


def time_steps(solver, dt, steps):
    import torch
    stream = solver.stream()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    solver.step(dt, steps)
    e1.record(stream)
    solver.sync()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / 1e3


def cpu_baseline(n, stages=2):
    """The reference's generated OPS solver (oracle/_ref/tgv_teno5, -O3 OpenMP) on the host
    cores: seconds per RK stage on the full n^3 workload, from its per-stage timestamps."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import harness
    cores = os.cpu_count() or 1
    if not harness.ref_available("tgv_teno5"):
        return None
    env = {"OSB_NP0": n, "OSB_NP1": n, "OSB_NP2": n, "OSB_NITER": 10}
    r = harness.run_ref("tgv_teno5", env=env, stop_after_rk=stages, threads=cores, fast=True, dump=False)
    t = r["_rk_times"]
    per_stage = (t[-1] - t[1]) / (len(t) - 2) if len(t) > 2 else (t[-1] - t[0])
    rate = n ** 3 / per_stage / 1e6
    return {"value": rate, "unit": UNIT, "cores": cores, "kind": "reference",
            "sample": "%d RK stages of the %d^3 TENO5 TGV with the reference's generated OPS solver (OpenMP, "
                      "-O3); rate from stage %d..%d timestamps" % (stages, n, 2, stages)}


def cpu_reference_rate(case, env, points, stages, what):
    """The reference's generated OPS solver for `case` (oracle/_ref/<case>, -O3, OpenMP on all
    host cores): Mpt-RK-stage/s from its per-stage timestamps after the first stage."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import harness
    cores = os.cpu_count() or 1
    if not harness.ref_available(case):
        return None
    r = harness.run_ref(case, env=dict(env, OSB_NITER=stages // 3 + 2), stop_after_rk=stages, threads=cores,
                        fast=True, dump=False)
    t = r["_rk_times"]
    per_stage = (t[-1] - t[1]) / (len(t) - 2)
    return {"value": points / per_stage / 1e6, "unit": UNIT, "cores": cores, "kind": "reference",
            "sample": "%d RK stages of %s with the reference's generated OPS solver (OpenMP, -O3); rate from "
                      "the stage timestamps after the first" % (stages, what)}


def cpu_port_rate(spec_q, dt, steps, what):
    """The oracle (the C restatement, -O2, OpenMP over its per-point loops) on a bounded sample:
    Mpt-RK-stage/s over `steps` whole steps of the block (spec, q)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import harness
    from opensbli_gb300 import abi, problems
    spec, q = spec_q
    ob = harness.OracleBlocks([(spec, q)])
    ob.apply_bc()
    t0 = time.perf_counter()
    ob.step(abi.RK_LOW_STORAGE, problems.RK3_LS_A, problems.RK3_LS_B, dt, steps)
    secs = time.perf_counter() - t0
    return {"value": spec.npoints * 3 * steps / secs / 1e6, "unit": UNIT, "cores": os.cpu_count() or 1,
            "kind": "port",
            "sample": "%d whole steps (3 RK stages + filter) of %s with the oracle (C restatement of the "
                      "reference path; its residual and update loops on all host cores with OpenMP, the filter "
                      "serial)" % (steps, what)}


def reference_arm(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import harness
    if not harness.ref_available("tgv_teno5"):
        print(json.dumps({"impl": "reference", "unavailable": "generated reference sources (oracle/_ref) missing"}))
        return 0
    n = args.size
    cores = os.cpu_count() or 1
    total = args.warmup + args.steps
    env = {"OSB_NP0": n, "OSB_NP1": n, "OSB_NP2": n, "OSB_NITER": total + 2}
    # one "step" of this arm = one RK stage of the n^3 workload (a bounded sample of a step)
    r = harness.run_ref("tgv_teno5", env=env, stop_after_rk=total, threads=cores, fast=True, dump=False,
                        timeout=3600)
    t = r["_rk_times"]  # start, then one stamp per stage
    timed = t[args.warmup + 1:]
    secs = timed[-1] - t[args.warmup]
    k = len(timed)
    rate = n ** 3 * k / secs / 1e6
    line = {"metric": METRIC, "value": rate, "unit": UNIT, "n_gpus": 0, "steps": k, "warmup": args.warmup,
            "ms_per_step": secs / k * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (analytic TGV initial condition)", "impl": "reference",
            "config": {"workload": "supersonic TGV %d^3 TENO5-Roe + central-4 viscous, RK-LS3; one step = one RK "
                                   "stage (bounded sample)" % n, "l2": "inputs larger than L2"},
            "cpu_baseline": {"value": rate, "unit": UNIT, "cores": cores, "kind": "reference",
                             "sample": "%d RK stages of the %d^3 workload" % (k, n)},
            "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def our_arm(args):
    import torch
    from opensbli_gb300 import abi, problems
    from opensbli_gb300.solver import Solver

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    n = args.size
    spec, q, dt = make_problem(n)
    pts = spec.npoints
    s32 = Solver([(spec, q)], precision="fp32", rk="ls3", device=local, graphs=True)
    s32.apply_bc()
    from opensbli_gb300 import autotune
    if args.fuse == "auto":
        sched, _ = autotune.tune(s32, dt, steps=2, warmup=1, cache=None)
    else:
        sched = dict(s32.schedule()[1], mode=abi.SCHED_PER_BLOCK, fuse_update=int(args.fuse), variant=args.variant)
        autotune.apply(s32, sched)
    log("schedule %s" % json.dumps(sched))
    s32.step(dt, args.warmup)
    s32.sync()
    log("warmup done")

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    launches0 = s32.launches()
    clocks = ClockSampler(local)
    clocks.start()
    barrier()
    secs = time_steps(s32, dt, args.steps)
    barrier()
    clk = clocks.stop()
    launches = s32.launches() - launches0
    log("timed done")
    if world > 1:
        from opensbli_gb300.replicas import max_over_ranks
        secs = max_over_ranks(secs)
    value = world * pts * 3 * args.steps / secs / 1e6

    # per-kernel times (CUDA events per launch on the context stream) over one more step
    s32.timing(True)
    s32.step(dt, 1)
    rep = s32.timing_report()
    s32.timing(False)
    log("kernel timing done")
    tot = sum(v[0] for v in rep.values()) or 1.0
    dom = max(rep, key=lambda k: rep[k][0])
    dom_ms = rep[dom][0] / max(rep[dom][1], 1)
    fused = rep["rk_update"][1] == 0
    alg_bytes_pt = kernel_bytes(fused)[dom]
    alg_bytes = alg_bytes_pt * pts
    hbm, peak_kind = measured_peaks()
    achieved = alg_bytes / (dom_ms * 1e-3) / 1e9
    step_bytes_gbs = BYTES_PER_PT_STAGE * pts * 3 * args.steps / secs / 1e9
    traffic = measured_traffic(dom, fused)
    if traffic is not None:
        traffic *= pts

    fp32_peak, fp64_peak = probe_fp(local)
    log("probe done")

    # FP64 parity path on the same workload, and the FP32-vs-FP64 error after the same steps
    fp64 = None
    err = None
    if not args.no_fp64 and rank == 0:
        s64 = Solver([(spec, q)], precision="fp64", rk="ls3", device=local, graphs=True)
        s64.apply_bc()
        s64.step(dt, 1)
        s64.sync()
        n64 = 1
        t64 = time_steps(s64, dt, n64)
        fp64 = pts * 3 * n64 / t64 / 1e6
        a = Solver([(spec, q)], precision="fp32", rk="ls3", device=local, graphs=True)
        a.apply_bc()
        a.step(dt, 1 + n64)
        qa = a.state(0)
        qb = s64.state(0)
        sl = spec.interior()
        err = {}
        for v, name in ((0, "rho"), (4, "rhoE")):
            d = qa[v][sl] - qb[v][sl]
            err[name] = {"rel_l2": float(np.linalg.norm(d) / np.linalg.norm(qb[v][sl])),
                         "rel_linf": float(np.max(np.abs(d)) / np.max(np.abs(qb[v][sl])))}
        ke_a = a.reduce(abi.RED_KE)
        ke_b = s64.reduce(abi.RED_KE)
        err["ke_rel"] = abs(ke_a - ke_b) / abs(ke_b)
        err["steps"] = 1 + n64
        a.close()
        s64.close()
        log("fp64 done")

    # end to end through the public API with pinned host buffers: H2D state, one RK step, D2H state
    host_q = torch.empty(s32.q[0].shape, dtype=torch.float64, pin_memory=True)
    host_q.copy_(torch.from_numpy(np.stack(q)))
    host_out = torch.empty_like(host_q, pin_memory=True)
    stream = s32.stream()
    e2e_steps = max(1, min(args.steps, 5))
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    parts = [0.0, 0.0, 0.0]
    # untimed warm-up rounds: the first transfers from a freshly pinned buffer run at a
    # fraction of the link rate
    for _ in range(max(1, min(args.warmup, 3))):
        with torch.cuda.stream(stream):
            s32.q[0].copy_(host_q, non_blocking=True)
        s32.apply_bc()
        s32.step(dt, 1)
        with torch.cuda.stream(stream):
            host_out.copy_(s32.q[0], non_blocking=True)
        s32.sync()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        ev[0].record(stream)
        with torch.cuda.stream(stream):
            s32.q[0].copy_(host_q, non_blocking=True)
        ev[1].record(stream)
        s32.apply_bc()
        s32.step(dt, 1)
        ev[2].record(stream)
        with torch.cuda.stream(stream):
            host_out.copy_(s32.q[0], non_blocking=True)
        ev[3].record(stream)
        s32.sync()
        for k in range(3):
            parts[k] += ev[k].elapsed_time(ev[k + 1])
    t_e2e = time.perf_counter() - t0
    log("e2e serial per step: H2D %.2f ms, step %.2f ms, D2H %.2f ms, wall %.2f ms"
        % tuple([x / e2e_steps for x in parts] + [t_e2e / e2e_steps * 1e3]))
    e2e_serial = world * pts * 3 * e2e_steps / t_e2e / 1e6
    # the same through osb_step_requests: every step still copies its state in from pinned
    # host memory and its result back, the copies of the next and previous step overlapping
    # this one's kernels on two copy streams
    nreq = max(3, min(args.steps, 10))
    outs = [host_out, torch.empty_like(host_q, pin_memory=True)]
    s32.step_requests([host_q] * 2, outs, dt, 1)  # staging buffers, copy streams
    torch.cuda.synchronize()
    # three timed calls (each ends with its copies and kernels complete), the median kept: the
    # host memory behind the copies is shared with other jobs, and a stall of it during a single
    # call would otherwise set the figure
    t_reqs = []
    for _ in range(3):
        t0 = time.perf_counter()
        s32.step_requests([host_q] * nreq, [outs[r & 1] for r in range(nreq)], dt, 1)
        t_reqs.append(time.perf_counter() - t0)
    t_req = sorted(t_reqs)[1]
    e2e_value = world * pts * 3 * nreq / t_req / 1e6
    e2e_calls = [t / nreq * 1e3 for t in t_reqs]
    log("e2e pipelined: %d steps, %.2f ms per step (median of %s; serial %.2f)"
        % (nreq, t_req / nreq * 1e3, ", ".join("%.2f" % t for t in e2e_calls), t_e2e / e2e_steps * 1e3))
    nbytes = host_q.numel() * 8
    # the pinned buffers were used on the solver's stream: release them before the stream goes
    torch.cuda.synchronize()
    del host_q, host_out, outs
    s32.close()
    del s32

    cpu = None
    log("e2e done")
    if not args.no_cpu and rank == 0 and world == 1:
        try:
            cpu = cpu_baseline(n)
        except Exception as ex:  # the baseline is reported, not required
            cpu = {"value": None, "unit": UNIT, "cores": os.cpu_count(), "kind": "reference",
                   "sample": "failed: %s" % str(ex)[:200]}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": secs / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 residual / f64 state",
            "data": "synthetic (analytic TGV initial condition, dt from CFL %.1f at t=0 = %.6g)" % (CFL, dt),
            "config": {"workload": "supersonic TGV %d^3, M=%.2f, Re=1600, TENO5 (Roe) + central-4 viscous, "
                                   "RK-LS3, periodic" % (n, MINF),
                       "points": pts, "stages_per_step": 3,
                       "l2": "inputs larger than L2 (752 MB state), no flush"},
            "fp64": {"value": fp64, "unit": UNIT,
                     "fp32_over_fp64": (value / world / fp64) if fp64 else None},
            "error_vs_fp64": err,
            "error_vs_fp64_1000_steps": ACCURACY_1000,
            "clocks": clk,
            "gpu_launches": launches,
            "schedule": sched,
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                         "frac": achieved / hbm, "traffic": traffic, "peak_kind": peak_kind,
                         "per_launch_ms": dom_ms, "share": rep[dom][0] / tot,
                         "algorithmic_bytes_per_point": alg_bytes_pt,
                         "traffic_source": "constant: DRAM bytes per point of this kernel from the ncu capture in "
                                           "profiles/dram_traffic_tgv_fp32.txt, times the points; not measured "
                                           "in this run",
                         "note": "the reconstruction sweeps are FP32-pipe bound; compute roof below"},
            "compute": {"fp32_peak_tflops": fp32_peak, "fp64_peak_tflops": fp64_peak},
            "step_hbm_gbs_at_160B": step_bytes_gbs,
            "kernel_ms_per_step": {k: v[0] for k, v in rep.items()},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
                    "api": "osb_step_requests (copies of the neighbouring steps overlap each step's kernels)",
                    "pipelined_calls_ms_per_step": e2e_calls, "serial_value": e2e_serial},
            "cpu_baseline": cpu,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def _errors(spec, qa, qb):
    sl = spec.interior()
    out = {}
    for v, name in ((0, "rho"), (spec.nvars - 1, "rhoE")):
        d = qa[v][sl] - qb[v][sl]
        out[name] = {"rel_l2": float(np.linalg.norm(d) / np.linalg.norm(qb[v][sl])),
                     "rel_linf": float(np.max(np.abs(d)) / np.max(np.abs(qb[v][sl])))}
    return out


def _merge_errors(per_block):
    """Worst relative error over blocks (L2 over the union of points)."""
    out = {}
    for name in ("rho", "rhoE"):
        out[name] = {"rel_l2": max(e[name]["rel_l2"] for e in per_block),
                     "rel_linf": max(e[name]["rel_linf"] for e in per_block)}
    return out


def secondary_arm(args):
    """sod / tgv64 / kh_ensemble / curv4 / c4w5 / tvd / shock / channel / tcf workloads: FP32-residual throughput (whole batch per step), the FP64
    per-block path beside it, the FP32-vs-FP64 error after the timed steps' count, launches."""
    import torch
    from opensbli_gb300 import abi, autotune, problems
    from opensbli_gb300.solver import Solver

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    cpu = None
    if args.workload == "sod":
        blocks = [problems.sod(400)]
        dt = 2e-4
        rk = "ls3"
        work = "Sod shock tube, 400 points, WENO5-JS (simple average), RK-LS3, zero-gradient ends"
        bytes_pt = 4 * 3 * 8
        cpu_args = ("sod_weno5js", {"OSB_NP0": 400}, 400, 600, "the 400-point Sod case")
    elif args.workload == "tgv64":
        blocks = [problems.tgv(64, minf=0.1, scheme=abi.SCHEME_CENTRAL4)]
        dt = 3.385e-3
        rk = "ls3"
        work = "TGV 64^3, M=0.1, Re=1600, central-4 Feiereisen + viscous, RK-LS3, periodic"
        bytes_pt = 4 * 5 * 8
        cpu_args = ("tgv_central", {"OSB_NP0": 64, "OSB_NP1": 64, "OSB_NP2": 64}, 64 ** 3, 12, "the 64^3 central TGV")
    elif args.workload == "kh_ensemble":
        blocks = problems.kh_ensemble(args.ensemble, seed=0)
        dt = 2e-4
        rk = "ls3"
        work = ("%d Kelvin-Helmholtz 2D instances, sizes drawn by seed 0 from {128,192,256,384,512}^2, "
                "WENO5-Z (Roe), RK-LS3, periodic" % args.ensemble)
        bytes_pt = 4 * 8 * 4 + 2 * 4 * 4  # q, rk read+write FP64 (4 vars) + FP32 state in/out
        cpu_args = ("kh_weno5z", {"OSB_NP0": 320, "OSB_NP1": 320}, 320 ** 2, 12,
                    "one 320^2 Kelvin-Helmholtz instance (the ensemble's mean size)")
    elif args.workload == "c4w5":
        n = args.size
        blocks = [problems.tgv_filtered(n)]
        dt = problems.filtered_dt(n)
        rk = "ls3"
        work = ("Central4-WENO5 benchmark TGV %d^3, M=1.25, Re=1600, central-4 KGP + Sutherland viscous, "
                "RK-LS3, non-linear WENO3-Z filter (Ducros 0.05) after every step, periodic" % n)
        bytes_pt = 4 * 5 * 8
        cpu_args = None
    elif args.workload == "shock":
        # the app as written: its own HLLC-LM flux from WENO5-Z states and its SSP RK3
        blocks = [problems.shock_reflection(457, 255, flux_type=abi.FLUX_HLLC_LM)]
        dt = 0.1
        rk = (abi.RK_LOW_STORAGE, problems.RK3_SSP_A, problems.RK3_SSP_B)
        work = ("2D inviscid shock reflection 457 x 255 (350 x 115, M=2), HLLC-LM flux from WENO5-Z states (simple "
                "average), SSP RK3, Dirichlet inlet and top, extrapolation outlet, symmetry wall, dt 0.1 as the app")
        bytes_pt = 4 * 4 * 8
        cpu_args = ("shock_reflection_hllc", {"OSB_NP0": 457, "OSB_NP1": 255, "OSB_DT": 0.1}, 457 * 255, 30,
                    "the 457 x 255 shock reflection with the app's HLLC-LM flux and SSP RK3")
    elif args.workload == "channel":
        blocks = [problems.channel_iso((256, 257, 128))]
        dt = 2e-4
        rk = "ls3"
        work = ("3D channel 256 x 257 x 128 between isothermal no-slip walls (Twall 1), M=0.5, Re=100, TENO5 (Roe) + "
                "central-4 viscous terms with the Carpenter closures at the walls, RK-LS3, periodic x and z")
        bytes_pt = 4 * 5 * 8
        cpu_args = ("channel_iso", {"OSB_NP0": 64, "OSB_NP1": 65, "OSB_NP2": 32, "OSB_DT": 2e-4}, 64 * 65 * 32, 12,
                    "a 64 x 65 x 32 channel of the reference's generated solver (the same discretisation)")
    elif args.workload == "tcf":
        blocks = [problems.channel_tcf((129, 129, 129))]
        dt = 2e-4
        rk = (abi.RK_LOW_STORAGE, problems.RK3_SSP_A, problems.RK3_SSP_B)
        work = ("the TENO turbulent-channel app's discretisation at its 129^3: TENO6 (Roe) + central-4 viscous "
                "terms with mu = T^0.7, forcing c = (-1, 0, 0), isothermal walls on the tanh-stretched y grid "
                "(stretch 1.7), Re 190.71, Minf 0.0955, SSP RK3, dt 2e-4 as the app")
        bytes_pt = 4 * 5 * 8
        cpu_args = ("channel_tcf", {"OSB_NP0": 64, "OSB_NP1": 65, "OSB_NP2": 32, "OSB_DT": 2e-4}, 64 * 65 * 32, 12,
                    "a 64 x 65 x 32 block of the reference's generated solver of the app's discretisation")
    elif args.workload == "tvd":
        n = args.size
        blocks = [problems.tgv_tvd(n, kappa=1.25)]
        dt = 0.0005 * 256 / n
        rk = "ls3"
        work = ("TGV %d^3 of the TGV app's TVD branch, M=1.25, Re=1600, central-4 KGP + Sutherland viscous, "
                "RK-LS3, non-linear TVD filter (kappa_TVD 1.25) after every step, periodic" % n)
        bytes_pt = 4 * 5 * 8
        cpu_args = ("tgv_kgp_tvd", {"OSB_NP0": 64, "OSB_NP1": 64, "OSB_NP2": 64, "OSB_KAPPA_TVD": 1.25,
                                    "OSB_DT": 0.0005 * 4}, 64 ** 3, 7,
                    "the 64^3 TVD-filtered TGV (two whole steps with their filters)")
    else:
        blocks = problems.curvilinear_multiblock_3d(seed=0)
        dt = problems.multiblock_cfl_dt(blocks, CFL)
        rk = "ls3"
        work = ("4-block 3D curvilinear Euler (512x256x32, 384x256x32, 512x192x32, 256x256x32), TENO5 (Roe), "
                "interfaces + periodic, Mach 0.7 + Gaussian pulse, RK-LS3, CFL %.1f" % CFL)
        bytes_pt = 4 * 5 * 8 + 10 * 8  # fused stage plus the ten FP64 metric arrays read
        cpu_args = ("curv3d_teno5", {"OSB_NP0": 256, "OSB_NP1": 256, "OSB_NP2": 32}, 256 * 256 * 32, 6,
                    "a 256x256x32 block of the reference's generated 3D curvilinear TENO5 solver (MetricsEquation "
                    "+ LFTeno(5), RK-LS3; the 4-block case's discretisation on one block of its sizes)")
    pts = sum(b[0].npoints for b in blocks)
    log("problem ready: %d blocks, %d points" % (len(blocks), pts))
    if not args.no_cpu:
        try:
            if args.workload == "c4w5":
                # the shipped solver's sources are not available to build on this host: the oracle
                # (pinned to it at 1e-11) times a bounded 48^3 sample
                cpu = cpu_port_rate(problems.tgv_filtered(48), problems.filtered_dt(48), 2, "the 48^3 filtered TGV")
            else:
                cpu = cpu_reference_rate(*cpu_args)
        except Exception as ex:  # the baseline is reported, not required
            cpu = {"value": None, "unit": UNIT, "kind": "reference", "sample": "failed: %s" % str(ex)[:200]}
        log("cpu baseline %s" % json.dumps(cpu))
    s32 = Solver(blocks, precision="fp32", rk=rk, device=local)
    s32.apply_bc()
    tuned = None
    if args.workload == "kh_ensemble" and not args.no_tune:
        best, trials = autotune.tune(s32, dt, steps=2, warmup=1, cache=autotune.DEFAULT_CACHE)
        tuned = {"schedule": best, "trials": len(trials),
                 "per_block_ms": next((t for t, c in trials if c["mode"] == abi.SCHED_PER_BLOCK), None),
                 "best_ms": min((t for t, _ in trials), default=None)}
        log("autotune: %s" % json.dumps(tuned))
    mode, sched = s32.schedule()
    s32.step(dt, args.warmup)
    s32.sync()
    launches0 = s32.launches()
    clocks = ClockSampler(local)
    clocks.start()
    secs = time_steps(s32, dt, args.steps)
    clk = clocks.stop()
    launches = s32.launches() - launches0
    value = pts * 3 * args.steps / secs / 1e6
    s32.timing(True)
    s32.step(dt, 1)
    rep = s32.timing_report()
    s32.timing(False)
    dom = max(rep, key=lambda k: rep[k][0])
    dom_ms = rep[dom][0] / max(rep[dom][1], 1)
    hbm, peak_kind = measured_peaks()
    launches_per_stage = rep[dom][1] / 3.0
    spec0 = blocks[0][0]
    table = kernel_bytes(rep["rk_update"][1] == 0, nv=spec0.nvars, ndim=spec0.ndim,
                         curvilinear=len(blocks[0]) > 2 and blocks[0][2] is not None,
                         central_only=spec0.scheme == abi.SCHEME_CENTRAL4)
    if dom == "persistent_stage":
        dom_bytes_pt = bytes_pt
    elif dom in ("flux_x", "flux_y", "flux_z", "central", "rk_update"):
        dom_bytes_pt = table[dom]
    else:
        dom_bytes_pt = None
    # bytes of one launch: every block's points, over the launches of one stage of that family
    achieved = (dom_bytes_pt * pts / launches_per_stage / (dom_ms * 1e-3) / 1e9) if dom_bytes_pt else None
    # FP64 per-block path and the error after the same number of steps from the same state
    s64 = Solver(blocks, precision="fp64", rk=rk, device=local)
    s64.apply_bc()
    s64.step(dt, 1)
    s64.sync()
    t64 = time_steps(s64, dt, 1)
    fp64 = pts * 3 / t64 / 1e6
    s64.close()
    nerr = 3
    a = Solver(blocks, precision="fp32", rk=rk, device=local)
    if tuned:
        autotune.apply(a, tuned["schedule"])
    a.apply_bc()
    a.step(dt, nerr)
    b = Solver(blocks, precision="fp64", rk=rk, device=local)
    b.apply_bc()
    b.step(dt, nerr)
    errs = [_errors(blk[0], a.state(i), b.state(i)) for i, blk in enumerate(blocks)]
    ke_a, ke_b = a.reduce(abi.RED_KE), b.reduce(abi.RED_KE)
    a.close()
    b.close()
    err = _merge_errors(errs)
    err["ke_rel"] = abs(ke_a - ke_b) / abs(ke_b)
    err["steps"] = nerr
    s32.close()
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": secs / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 residual / f64 state", "data": "synthetic",
            "config": {"workload": work, "points": pts, "blocks": len(blocks),
                       "schedule": "persistent" if mode == abi.SCHED_PERSISTENT else "per-block",
                       "l2": "inputs larger than L2, no flush"},
            "autotune": tuned, "fp64": {"value": fp64, "unit": UNIT, "fp32_over_fp64": value / fp64},
            "error_vs_fp64": err, "clocks": clk, "gpu_launches": launches, "cpu_baseline": cpu,
            "kernel_ms_per_step": {k: v[0] for k, v in rep.items() if v[1]},
            "schedule": sched,
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                         "frac": achieved / hbm if achieved else None, "peak_kind": peak_kind,
                         "per_launch_ms": dom_ms, "algorithmic_bytes_per_point": dom_bytes_pt,
                         "traffic": None},
            "step_hbm_gbs_at_fused_bytes": bytes_pt * pts * 3 * args.steps / secs / 1e9}
    print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return reference_arm(args)
    if args.workload != "tgv":
        return secondary_arm(args)
    return our_arm(args)


if __name__ == "__main__":
    sys.exit(main())
