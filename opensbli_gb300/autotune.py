"""Autotuner of the stage schedule (osb_set_schedule).

For a solver holding its blocks, times every candidate schedule -- per-block launches with and
without the RK update fused into the last residual kernel and with each x-sweep segment length
(osb_set_variant: the wave-model length, whole rows, 64, 32, 16, 48 points), and the persistent
fused stage over
tile heights, resident CTAs per SM, static or dynamic tile claiming and tile orders -- on the
caller's own workload (CUDA-graph replays timed with CUDA events on the
solver's stream), restores the state after every trial, applies the fastest schedule and caches
it in a JSON file keyed by the device, the precision and the blocks' shapes and schemes, so a
later solver with the same workload picks it up without timing.

    from opensbli_gb300 import autotune
    best, trials = autotune.tune(solver, dt)

The reference's counterpart is OPS's tiling configuration (OPS_TILING with OPS_TILESIZE_X /
_Y, set by hand per machine); here the knobs are measured per workload.
"""
import json
import os
import tempfile

from . import abi

DEFAULT_CACHE = os.environ.get("OSB_AUTOTUNE_CACHE",
                               os.path.join(os.path.expanduser("~"), ".cache", "opensbli_gb300", "autotune.json"))


def candidates(persistent):
    """Candidate schedules: the per-block path, plus the persistent stage's knob grid."""
    out = [{"mode": abi.SCHED_PER_BLOCK, "tile_y": 16, "ctas_per_sm": 2, "dynamic": 1, "order": 0, "fuse_update": f,
            "variant": v} for f in (1, 0) for v in range(6)]
    if persistent:
        for ty in (8, 16, 32):
            for cps in (1, 2, 3, 4):
                for dyn in (1, 0):
                    for order in (0, 1, 2):
                        out.append({"mode": abi.SCHED_PERSISTENT, "tile_y": ty, "ctas_per_sm": cps,
                                    "dynamic": dyn, "order": order, "fuse_update": 1, "variant": 0})
    return out


def apply(solver, cand):
    """Apply one candidate: the osb_schedule fields plus the x-sweep variant."""
    sched = {k: v for k, v in cand.items() if k != "variant"}
    solver.set_schedule(**sched)
    solver.set_variant(cand.get("variant", 0))


def signature(solver):
    torch = solver.torch
    dev = torch.cuda.get_device_name(solver.device)
    blocks = [[s.ndim, list(s.size[:s.ndim]), s.scheme, s.averaging, s.viscous,
               [list(b) for b in s.bc]] for s in solver.specs]
    return json.dumps({"device": dev, "precision": solver.precision, "rk": solver.rk_kind, "blocks": blocks},
                      sort_keys=True)


def _load(cache):
    try:
        with open(cache) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(cache, table):
    d = os.path.dirname(cache)
    if d:
        os.makedirs(d, exist_ok=True)
    fd, tmp = tempfile.mkstemp(dir=d or ".", prefix=".autotune")
    with os.fdopen(fd, "w") as f:
        json.dump(table, f, indent=1, sort_keys=True)
    os.replace(tmp, cache)


def time_schedule(solver, dt, steps, warmup):
    """Milliseconds per step of the solver's current schedule (graph replays, CUDA events on
    the solver's stream)."""
    torch = solver.torch
    solver.step(dt, warmup)
    solver.sync()
    st = solver.stream()
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    a.record(st)
    solver.step(dt, steps)
    b.record(st)
    solver.sync()
    return a.elapsed_time(b) / steps


def tune(solver, dt, steps=3, warmup=1, cache=DEFAULT_CACHE, force=False, cands=None):
    """Pick the fastest schedule for the solver's workload; returns (schedule, trials) where
    trials is [(ms per step, schedule)] (empty when the cache answered)."""
    key = signature(solver)
    table = _load(cache) if cache else {}
    if not force and key in table:
        best = table[key]["schedule"]
        apply(solver, best)
        return best, []
    torch = solver.torch
    solver.sync()
    saved_q = [q.clone() for q in solver.q]
    saved_rk = [r.clone() for r in solver.rk]
    torch.cuda.synchronize(solver.device)
    persistent_ok = True
    try:
        solver.set_schedule(mode=abi.SCHED_PERSISTENT)
    except abi.OSBError:
        persistent_ok = False
    trials = []
    for cand in (cands or candidates(persistent_ok)):
        try:
            apply(solver, cand)
        except abi.OSBError:
            continue
        for q, s in zip(solver.q, saved_q):
            q.copy_(s)
        for r, s in zip(solver.rk, saved_rk):
            r.copy_(s)
        torch.cuda.synchronize(solver.device)
        trials.append((time_schedule(solver, dt, steps, warmup), cand))
    for q, s in zip(solver.q, saved_q):
        q.copy_(s)
    for r, s in zip(solver.rk, saved_rk):
        r.copy_(s)
    torch.cuda.synchronize(solver.device)
    ms, best = min(trials, key=lambda t: t[0])
    apply(solver, best)
    solver.apply_bc()
    if cache:
        table = _load(cache)
        table[key] = {"schedule": best, "ms_per_step": ms}
        _store(cache, table)
    return best, trials
