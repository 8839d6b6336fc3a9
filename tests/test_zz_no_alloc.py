"""osb_stage_noalloc: one RK stage for callers that cannot allocate device memory.

The entry point keeps its residual workspace in a fixed-size static device array, so an
application that hands out all GPU memory from its own pool (or must not call cudaMalloc once
running) can still advance a block; it is checked here, through the C ABI, against the
context-based entry point (osb_stage) on two consecutive stages.  Collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

from opensbli_gb300 import abi, problems

pytestmark = pytest.mark.gpu

TOL = 1e-12  # same FP64 tolerance as the other parity tests


def _rel(a, b):
    return float(np.max(np.abs(a - b))) / max(float(np.max(np.abs(b))), 1e-300)


def test_stage_noalloc_matches_stage(built_lib):
    import torch
    from opensbli_gb300.solver import Solver

    spec, q = problems.tgv(20, minf=1.25, scheme=abi.SCHEME_TENO5, averaging=abi.AVG_ROE)
    dt = 1e-3
    A, B = problems.RK3_LS_A, problems.RK3_LS_B

    # existing entry point: a context with its own (cudaMalloc'd) workspace
    s = Solver([(spec, q)], precision="fp64", rk="ls3")
    s.apply_bc()
    s.stage(0, dt)
    s.stage(1, dt)
    ref_q = s.state(0)
    ref_rk = s.rk_register(0)
    s.close()

    # allocation-free entry point on caller-owned arrays
    lib = abi.load_library()
    dev = torch.device("cuda", 0)
    qd = torch.from_numpy(np.ascontiguousarray(np.stack(q))).to(dev)
    rkd = torch.zeros_like(qd)
    d = abi.make_desc(spec, [qd[v].data_ptr() for v in range(spec.nvars)],
                      [rkd[v].data_ptr() for v in range(spec.nvars)])
    torch.cuda.synchronize()
    for stage in range(2):
        rc = lib.osb_stage_noalloc(ctypes.byref(d), abi.RK_LOW_STORAGE, A[stage], B[stage], dt, None)
        assert rc == abi.OSB_OK, abi.last_error(lib)
    torch.cuda.synchronize()
    got_q = qd.cpu().numpy()
    got_rk = rkd.cpu().numpy()
    sl = spec.interior()
    for v in range(spec.nvars):
        assert _rel(got_q[v][sl], ref_q[v][sl]) < TOL, v
        assert _rel(got_rk[v][sl], ref_rk[v][sl]) < TOL, v


def test_stage_noalloc_rejects_oversized_block(built_lib):
    lib = abi.load_library()
    spec, _ = problems.tgv(minf=1.25, scheme=abi.SCHEME_TENO5, averaging=abi.AVG_ROE, sizes=(128, 128, 128))
    fake = [1] * spec.nvars  # never dereferenced: the size check comes first
    d = abi.make_desc(spec, fake, fake)
    rc = lib.osb_stage_noalloc(ctypes.byref(d), abi.RK_LOW_STORAGE, 0.0, 1.0 / 3.0, 1e-3, None)
    assert rc == abi.OSB_EINVAL
    msg = abi.last_error(lib)
    assert "static workspace" in msg and str(abi.NOALLOC_MAX_DOUBLES) in msg
