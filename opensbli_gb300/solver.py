"""Device-side engine: owns the FP64 state of every block in HBM (torch tensors used only as
allocations) and drives libosb_gb300 through its C ABI.

This is the runtime the backend (``backend.GB300Backend``) hands an OpenSBLI algorithm to,
and what tests and the benchmark call directly with ``BlockSpec`` objects.  There is no CPU
path: constructing a ``Solver`` without the CUDA library or without a GPU raises.
"""
import ctypes

import numpy as np

from . import abi
from .problems import RK3_LS_A, RK3_LS_B, RK3_SBLI_NEW, RK3_SBLI_OLD


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise abi.OSBError("no CUDA device: the GB300 path has no CPU fallback")
    return torch


class Solver:
    """Advance one or more blocks with the GB300 kernels.

    specs_states: list of (BlockSpec, [nv arrays in OPS layout]) pairs, or triples whose third
        item is the list of 10 metric arrays of a curvilinear block (osb_block_desc.metric
        order: D_di at 3*d + i, det J at 9; None where unused; numpy arrays or CUDA tensors).
        A spec marked curvilinear must come with its metric arrays.
    precision: "fp64" (parity path) or "fp32" (FP32 residual, FP64 state).
    rk: "ls3" (RungeKuttaLS(3)), "sbli3" (RungeKutta(3)) or (kind, A, B).
    """

    def __init__(self, specs_states, precision="fp64", rk="ls3", device=0, graphs=True, rkold=None):
        torch = _torch()
        self.torch = torch
        self.lib = abi.load_library()
        self.device = torch.device("cuda", device)
        self.precision = precision
        prec = abi.PREC_FP64 if precision == "fp64" else abi.PREC_FP32_RESIDUAL
        ctx = ctypes.c_void_p()
        abi.check(self.lib, self.lib.osb_ctx_create(device, prec, ctypes.byref(ctx)), "osb_ctx_create")
        self.ctx = ctx
        self.specs = []
        self.q = []
        self.rk = []
        self.met = []
        self._dirichlet = []
        self._ystretch = []
        self._descs = []
        try:
            for i, item in enumerate(specs_states):
                spec, state = item[0], item[1]
                met = item[2] if len(item) > 2 else None
                q = torch.empty((spec.nvars,) + spec.shape, dtype=torch.float64, device=self.device)
                q.copy_(torch.from_numpy(np.ascontiguousarray(np.stack([np.asarray(a, dtype=np.float64) for a in state]))))
                r = torch.zeros_like(q)
                if rkold is not None:
                    r.copy_(torch.from_numpy(np.ascontiguousarray(np.stack(rkold[i]))))
                self.specs.append(spec)
                self.q.append(q)
                self.rk.append(r)
                mt, mp = None, None
                if met is None and getattr(spec, "curvilinear", False):
                    raise abi.OSBError("block %d is curvilinear: its metric arrays must be given" % i)
                if met is not None:
                    for a in met:
                        if a is not None and tuple(a.shape) != tuple(spec.shape):
                            raise abi.OSBError("metric array of shape %s, block allocation is %s"
                                               % (tuple(a.shape), spec.shape))
                    mt = [None if a is None else
                          (a.to(device=self.device, dtype=torch.float64).contiguous() if torch.is_tensor(a) else
                           torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).to(self.device))
                          for a in met]
                    mp = [None if a is None else a.data_ptr() for a in mt]
                self.met.append(mt)
                dp = None
                if spec.dirichlet:
                    dt_ = {k: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).to(self.device)
                           for k, a in spec.dirichlet.items()}
                    self._dirichlet.append(dt_)
                    dp = {k: a.data_ptr() for k, a in dt_.items()}
                yp = None
                if spec.ystretch is not None:  # the library copies the rows at osb_block_add
                    ys = [torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).to(self.device)
                          for a in spec.ystretch]
                    self._ystretch.append(ys)
                    yp = [a.data_ptr() for a in ys]
                d = abi.make_desc(spec, [q[v].data_ptr() for v in range(spec.nvars)],
                                  [r[v].data_ptr() for v in range(spec.nvars)], mp, dp, yp)
                self._descs.append(d)
                bid = ctypes.c_int()
                torch.cuda.synchronize(self.device)
                abi.check(self.lib, self.lib.osb_block_add(self.ctx, ctypes.byref(d), ctypes.byref(bid)), "osb_block_add")
            self.set_rk(rk)
            abi.check(self.lib, self.lib.osb_set_graphs(self.ctx, 1 if graphs else 0), "osb_set_graphs")
        except Exception:
            self.close()
            raise

    # -- configuration -------------------------------------------------------------------
    def set_rk(self, rk):
        if rk == "ls3":
            kind, A, B = abi.RK_LOW_STORAGE, RK3_LS_A, RK3_LS_B
        elif rk == "sbli3":
            kind, A, B = abi.RK_SBLI3, RK3_SBLI_NEW, RK3_SBLI_OLD
        else:
            kind, A, B = rk
        self.rk_kind, self.A, self.B = kind, tuple(A), tuple(B)
        Aa = (ctypes.c_double * len(A))(*A)
        Bb = (ctypes.c_double * len(B))(*B)
        abi.check(self.lib, self.lib.osb_set_rk(self.ctx, kind, len(A), Aa, Bb), "osb_set_rk")

    def set_schedule(self, mode=abi.SCHED_AUTO, tile_y=16, ctas_per_sm=2, dynamic=1, order=0, fuse_update=1):
        """Stage schedule (osb_set_schedule): per-block launches or one persistent launch per
        stage, with the persistent stage's tiling knobs and the per-block path's RK fusion."""
        sc = abi.Schedule(mode, tile_y, ctas_per_sm, dynamic, order, fuse_update)
        abi.check(self.lib, self.lib.osb_set_schedule(self.ctx, ctypes.byref(sc)), "osb_set_schedule")

    def set_variant(self, variant):
        """Tiling variant of the x reconstruction sweep (osb_set_variant)."""
        abi.check(self.lib, self.lib.osb_set_variant(self.ctx, int(variant)), "osb_set_variant")

    def set_central_staging(self, bulk):
        """Plane staging of the FP32 central kernel: bulk copies (1) or register loads (0)."""
        abi.check(self.lib, self.lib.osb_set_central_staging(self.ctx, int(bulk)), "osb_set_central_staging")

    def schedule(self):
        """(resolved mode, settings dict) of osb_get_schedule."""
        mode = ctypes.c_int()
        sc = abi.Schedule()
        abi.check(self.lib, self.lib.osb_get_schedule(self.ctx, ctypes.byref(mode), ctypes.byref(sc)),
                  "osb_get_schedule")
        return mode.value, sc.as_dict()

    # -- time stepping -------------------------------------------------------------------
    def apply_bc(self):
        abi.check(self.lib, self.lib.osb_apply_bc(self.ctx), "osb_apply_bc")

    def step(self, dt, nsteps=1):
        abi.check(self.lib, self.lib.osb_step(self.ctx, float(dt), int(nsteps)), "osb_step")

    def step_requests(self, host_in, host_out, dt, nsteps=1):
        """Independent runs from host memory (osb_step_requests): request r copies its state
        from host_in[r], advances nsteps steps and leaves the result in host_out[r].  Each
        buffer is a pinned torch tensor (or anything with data_ptr()) holding every block's
        variables in block order, whole allocations (the shape of torch.cat of self.q), so the
        copies overlap the steps.  Returns when every result is in host memory."""
        n = len(host_in)
        if len(host_out) != n:
            raise ValueError("host_in and host_out differ in length")
        need = sum(q.numel() for q in self.q) * 8
        for b in list(host_in) + list(host_out):
            if b.numel() * b.element_size() != need:
                raise ValueError("request buffer of %d bytes, the blocks need %d" % (b.numel() * b.element_size(), need))
        vp = ctypes.c_void_p
        ins = (vp * max(n, 1))(*[b.data_ptr() for b in host_in])
        outs = (vp * max(n, 1))(*[b.data_ptr() for b in host_out])
        abi.check(self.lib, self.lib.osb_step_requests(self.ctx, n, ins, outs, float(dt), int(nsteps)),
                  "osb_step_requests")

    # -- checkpoint / restart (restart.py: the reference's restart content, .npz layout) ---
    def save_restart(self, path, iteration, simulation_time):
        """Write every block's FP64 state and RK register (whole allocations) with the
        iteration count and simulation time."""
        from . import restart
        self.sync()
        restart.write(path, self.specs, [[a.cpu().numpy() for a in q] for q in self.q],
                      [[a.cpu().numpy() for a in r] for r in self.rk], iteration, simulation_time)

    def load_restart(self, path):
        """Load state and RK register of every block from a restart file written for the same
        blocks; returns (iteration, simulation_time).  The next step continues exactly as the
        run that wrote the file."""
        from . import restart
        data = restart.read(path)
        restart.check_compatible(self.specs, data)
        self.sync()
        for q, r, blk in zip(self.q, self.rk, data["blocks"]):
            q.copy_(self.torch.from_numpy(np.ascontiguousarray(np.stack(blk["state"]))))
            r.copy_(self.torch.from_numpy(np.ascontiguousarray(np.stack(blk["register"]))))
        self.torch.cuda.synchronize(self.device)
        return data["iter"], data["simulation_time"]

    def stage(self, s, dt):
        abi.check(self.lib, self.lib.osb_stage(self.ctx, int(s), float(dt)), "osb_stage")

    def save_sbli(self):
        """Copy q into the RK register (the SBLI RK3 start-of-step save) for stage-level use."""
        for q, r in zip(self.q, self.rk):
            r.copy_(q)

    def sync(self, timeout_ms=600000):
        abi.check(self.lib, self.lib.osb_sync(self.ctx, int(timeout_ms)), "osb_sync")

    # -- outputs -------------------------------------------------------------------------
    def residual(self, ib=0):
        spec = self.specs[ib]
        out = self.torch.zeros_like(self.q[ib])
        ptrs = (ctypes.c_void_p * 5)(*([out[v].data_ptr() for v in range(spec.nvars)] + [None] * (5 - spec.nvars)))
        abi.check(self.lib, self.lib.osb_residual(self.ctx, ib, ptrs), "osb_residual")
        self.sync()
        return [out[v].cpu().numpy() for v in range(spec.nvars)]

    def reduce(self, what):
        out = ctypes.c_double()
        abi.check(self.lib, self.lib.osb_reduce(self.ctx, int(what), ctypes.byref(out)), "osb_reduce")
        return out.value

    def state(self, ib=0):
        self.sync()
        return [a.cpu().numpy() for a in self.q[ib]]

    def rk_register(self, ib=0):
        self.sync()
        return [a.cpu().numpy() for a in self.rk[ib]]

    def launches(self):
        n = ctypes.c_longlong()
        abi.check(self.lib, self.lib.osb_launch_count(self.ctx, ctypes.byref(n)), "osb_launch_count")
        return n.value

    def stream(self):
        s = ctypes.c_void_p()
        abi.check(self.lib, self.lib.osb_get_stream(self.ctx, ctypes.byref(s)), "osb_get_stream")
        return self.torch.cuda.ExternalStream(s.value, device=self.device)

    def timing(self, enable):
        abi.check(self.lib, self.lib.osb_timing(self.ctx, 1 if enable else 0), "osb_timing")

    def timing_report(self):
        """{family: (milliseconds, launches)} accumulated since the last report."""
        n = len(abi.KERNEL_FAMILIES)
        ms = (ctypes.c_double * n)()
        cnt = (ctypes.c_longlong * n)()
        abi.check(self.lib, self.lib.osb_timing_report(self.ctx, ms, cnt, n), "osb_timing_report")
        return {f: (ms[i], cnt[i]) for i, f in enumerate(abi.KERNEL_FAMILIES)}

    def close(self):
        if getattr(self, "ctx", None) is not None and self.ctx.value:
            self.lib.osb_ctx_destroy(self.ctx)
            self.ctx = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def device_metrics(spec, x, fill=abi.METRIC_EDGE, device=0):
    """Metric arrays of a curvilinear block computed on the GPU (osb_metrics) from its grid
    coordinates x[0..ndim-1] (OPS-layout arrays known at every allocated point, numpy or CUDA
    tensors): the 10 slots of osb_block_desc.metric as CUDA tensors (None where a 2D block has
    none).  fill = abi.METRIC_PERIODIC for a periodic block (interior, halos its images),
    abi.METRIC_EDGE otherwise (where the stencil fits, outer layers the nearest)."""
    torch = _torch()
    lib = abi.load_library()
    dev = torch.device("cuda", device)
    xs = [torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64) if isinstance(a, np.ndarray) else a,
                          dtype=torch.float64, device=dev).contiguous() for a in x]
    used = [0, 1, 3, 4, 9] if spec.ndim == 2 else list(range(10))
    met = [torch.empty(spec.shape, dtype=torch.float64, device=dev) if k in used else None for k in range(10)]
    d = abi.make_desc(spec, [0] * 5, [0] * 5)
    vp = ctypes.c_void_p
    xp = (vp * 3)(*([t.data_ptr() for t in xs] + [0] * (3 - len(xs))))
    mp = (vp * 10)(*[0 if m is None else m.data_ptr() for m in met])
    stream = torch.cuda.current_stream(dev).cuda_stream
    abi.check(lib, lib.osb_metrics(ctypes.byref(d), xp, mp, int(fill), vp(stream)), "osb_metrics")
    torch.cuda.synchronize(dev)
    return met

