"""osb_stage_noalloc: one RK stage for callers that cannot allocate device memory.

Some hosts of this solver cannot call cudaMalloc: an application that hands out all GPU memory
from its own pool allocator, or one that must not allocate once it is running (allocation can
synchronise the device or fail under memory pressure in the middle of a run).  The entry point
keeps its residual workspace in a fixed-size static device array instead, and the caller passes
its own state and RK arrays.  These tests call it through the C ABI and compare it with the
context-based entry point (osb_stage) on two consecutive stages, for a periodic 3D TENO5 block,
a 2D block with Dirichlet, symmetry and extrapolation faces, a channel between an isothermal
and an adiabatic wall, and the SBLI RK3 integrator.
Collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

from opensbli_gb300 import abi, problems

pytestmark = pytest.mark.gpu

TOL = 1e-12  # same FP64 tolerance as the other parity tests


def _rel(a, b):
    return float(np.max(np.abs(a - b))) / max(float(np.max(np.abs(b))), 1e-300)


def _filled_halos(spec, q):
    """The state with its halos zeroed and then filled by the block's boundary faces on a
    context (osb_apply_bc): the precondition of osb_stage_noalloc, met the way a caller would."""
    from opensbli_gb300.solver import Solver
    h = spec.halo
    z = []
    for a in q:
        b = np.zeros(spec.shape)
        sl = spec.interior()
        b[sl] = np.asarray(a)[sl]
        z.append(b)
    s = Solver([(spec, z)], precision="fp64", rk="ls3")
    s.apply_bc()
    out = s.state(0)
    s.close()
    assert all(np.all(np.isfinite(a)) for a in out), h
    return out


def _check(spec, q, rk, stages, dt):
    import torch
    from opensbli_gb300.solver import Solver

    kind, A, B = {"ls3": (abi.RK_LOW_STORAGE, problems.RK3_LS_A, problems.RK3_LS_B),
                  "ssp3": (abi.RK_LOW_STORAGE, problems.RK3_SSP_A, problems.RK3_SSP_B),
                  "sbli3": (abi.RK_SBLI3, problems.RK3_SBLI_NEW, problems.RK3_SBLI_OLD)}[rk]
    q0 = _filled_halos(spec, q)

    # existing entry point: a context with its own (cudaMalloc'd) workspace
    s = Solver([(spec, q0)], precision="fp64", rk=(kind, A, B))
    if kind == abi.RK_SBLI3:
        s.save_sbli()
    for st in stages:
        s.stage(st, dt)
    ref_q = s.state(0)
    ref_rk = s.rk_register(0)
    s.close()

    # allocation-free entry point on caller-owned arrays
    lib = abi.load_library()
    dev = torch.device("cuda", 0)
    qd = torch.from_numpy(np.ascontiguousarray(np.stack(q0))).to(dev)
    rkd = torch.zeros_like(qd)
    if kind == abi.RK_SBLI3:
        rkd.copy_(qd)  # the SBLI start-of-step save is the caller's
    dp = None
    keep = []
    if spec.dirichlet:
        keep = {k: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).to(dev)
                for k, a in spec.dirichlet.items()}
        dp = {k: a.data_ptr() for k, a in keep.items()}
    yp = None
    if spec.ystretch is not None:
        keep_ys = [torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in spec.ystretch]
        yp = [a.data_ptr() for a in keep_ys]
    d = abi.make_desc(spec, [qd[v].data_ptr() for v in range(spec.nvars)],
                      [rkd[v].data_ptr() for v in range(spec.nvars)], None, dp, yp)
    torch.cuda.synchronize()
    for st in stages:
        rc = lib.osb_stage_noalloc(ctypes.byref(d), kind, A[st], B[st], dt, None)
        assert rc == abi.OSB_OK, abi.last_error(lib)
    torch.cuda.synchronize()
    got_q = qd.cpu().numpy()
    got_rk = rkd.cpu().numpy()
    sl = spec.interior()
    for v in range(spec.nvars):
        assert _rel(got_q[v][sl], ref_q[v][sl]) < TOL, v
        assert _rel(got_rk[v][sl], ref_rk[v][sl]) < TOL, v
        # the faces were applied after the update, as osb_stage does
        assert _rel(got_q[v], ref_q[v]) < TOL, ("halos", v)
    del keep


def test_stage_noalloc_matches_stage(built_lib):
    spec, q = problems.tgv(20, minf=1.25, scheme=abi.SCHEME_TENO5, averaging=abi.AVG_ROE)
    _check(spec, q, "ls3", [0, 1], 1e-3)


def test_stage_noalloc_dirichlet_symmetry_extrapolation(built_lib):
    spec, q = problems.shock_reflection(sizes=(64, 32))
    rng = np.random.default_rng(3)
    q = [a * (1.0 + 1e-3 * rng.standard_normal(a.shape)) for a in q]
    _check(spec, q, "ssp3", [0, 1], 0.1)


def test_stage_noalloc_walls(built_lib):
    """Isothermal and adiabatic no-slip walls (y faces) with the Carpenter closures of the
    viscous terms: the wall kernels and the closure-aware central kernel on the noalloc path."""
    spec, q = problems.channel_iso((16, 17, 8), upper="adiabatic")
    rng = np.random.default_rng(5)
    q = [a * (1.0 + 1e-3 * rng.standard_normal(a.shape)) for a in q]
    _check(spec, q, "ls3", [0, 1], 1e-3)


def test_stage_noalloc_stretched_walls(built_lib):
    """The walls on the stretched wall-normal grid (osb_block_desc.ystretch rows on the device)."""
    spec, q = problems.channel_iso((16, 17, 8), stretch=1.7)
    rng = np.random.default_rng(6)
    q = [a * (1.0 + 1e-3 * rng.standard_normal(a.shape)) for a in q]
    _check(spec, q, "ls3", [0, 1], 1e-3)


def test_stage_noalloc_sbli3(built_lib):
    spec, q = problems.kh(sizes=(40, 36))
    _check(spec, q, "sbli3", [0, 1], 1e-3)


def test_stage_noalloc_refuses_interfaces_before_launching(built_lib):
    import torch
    lib = abi.load_library()
    spec, q = problems.tgv(12, minf=1.25, scheme=abi.SCHEME_TENO5, averaging=abi.AVG_ROE)
    spec.bc[0] = [abi.BC_INTERFACE, abi.BC_INTERFACE]
    spec.iface = [[(0, 0, 1, 0), (0, 0, 0, 0)], [None, None], [None, None]]
    dev = torch.device("cuda", 0)
    qd = torch.from_numpy(np.ascontiguousarray(np.stack(q))).to(dev)
    before = qd.clone()
    rkd = torch.zeros_like(qd)
    d = abi.make_desc(spec, [qd[v].data_ptr() for v in range(spec.nvars)],
                      [rkd[v].data_ptr() for v in range(spec.nvars)])
    rc = lib.osb_stage_noalloc(ctypes.byref(d), abi.RK_LOW_STORAGE, 0.0, 1.0 / 3.0, 1e-3, None)
    torch.cuda.synchronize()
    assert rc == abi.OSB_ENOTSUP
    assert "interface" in abi.last_error(lib)
    assert torch.equal(qd, before) and not torch.any(rkd)


def test_stage_noalloc_rejects_host_arrays(built_lib):
    lib = abi.load_library()
    spec, q = problems.tgv(12, minf=1.25, scheme=abi.SCHEME_TENO5, averaging=abi.AVG_ROE)
    host = [np.ascontiguousarray(a) for a in q]
    rk = [np.zeros_like(a) for a in q]
    d = abi.make_desc(spec, [a.ctypes.data for a in host], [a.ctypes.data for a in rk])
    rc = lib.osb_stage_noalloc(ctypes.byref(d), abi.RK_LOW_STORAGE, 0.0, 1.0 / 3.0, 1e-3, None)
    assert rc == abi.OSB_EINVAL
    assert "device memory" in abi.last_error(lib)


def test_stage_noalloc_rejects_oversized_block(built_lib):
    lib = abi.load_library()
    spec, _ = problems.tgv(minf=1.25, scheme=abi.SCHEME_TENO5, averaging=abi.AVG_ROE, sizes=(128, 128, 128))
    fake = [1] * spec.nvars  # never dereferenced: the size check comes first
    d = abi.make_desc(spec, fake, fake)
    rc = lib.osb_stage_noalloc(ctypes.byref(d), abi.RK_LOW_STORAGE, 0.0, 1.0 / 3.0, 1e-3, None)
    assert rc == abi.OSB_EINVAL
    msg = abi.last_error(lib)
    assert "static workspace" in msg and str(abi.NOALLOC_MAX_DOUBLES) in msg
