"""Parity at the benchmark configurations' own sizes (the other GPU tests use small blocks),
and the 3D curvilinear path against the reference's own generated solver.

* the 256^3 supersonic TGV (TENO5, Roe average, central viscous terms), one RK stage;
* the 64^3 low-Mach TGV with the central scheme, three stages;
* the 4-block curvilinear 3D case at its full block sizes (12.6 M points), three stages;
each FP64 GPU path against the oracle advanced from the same state (1e-12 relative, per
variable on its own scale); the persistent batched stage (FP32 residual) on one
Kelvin-Helmholtz instance of each ensemble size against the FP64 oracle after one step, at
the FP32-residual tolerance; and the 3D curvilinear TENO5 block against the golden states of
the reference's generated solver (its own metric arrays, 1, 3 and 30 stages).  The oracle runs
on the host cores (OpenMP), seconds per stage.
"""
import os

import numpy as np
import pytest

from opensbli_gb300 import abi, problems

from test_gpu_parity import state_errors

pytestmark = pytest.mark.gpu

LS = (abi.RK_LOW_STORAGE, problems.RK3_LS_A, problems.RK3_LS_B)
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _gpu(blocks, dt, stages=0, steps=0, precision="fp64", schedule=None):
    from opensbli_gb300.solver import Solver
    s = Solver(blocks, precision=precision, rk="ls3")
    if schedule is not None:
        s.set_schedule(**schedule)
    s.apply_bc()
    if steps:
        s.step(dt, steps)
    for st in range(stages):
        s.stage(st, dt)
    out = [s.state(i) for i in range(len(blocks))]
    s.close()
    return out


def _oracle(blocks, dt, stages=0, steps=0):
    import harness
    ob = harness.OracleBlocks(blocks)
    ob.apply_bc()
    if steps:
        ob.step(*LS, dt, steps)
    for st in range(stages):
        ob.stage(*LS, st, dt)
    return ob


def test_supersonic_tgv_256_one_stage(built_lib, oracle_lib):
    spec, q = problems.tgv(256, minf=1.25, scheme=abi.SCHEME_TENO5, averaging=abi.AVG_ROE)
    dt = problems.cfl_dt(spec, q, 0.5)
    got = _gpu([(spec, q)], dt, stages=1)[0]
    ob = _oracle([(spec, q)], dt, stages=1)
    errs = state_errors(spec, got, ob.q[0])
    assert max(errs) < 1e-12, errs


def test_central_tgv_64_three_stages(built_lib, oracle_lib):
    spec, q = problems.tgv(64, minf=0.1, scheme=abi.SCHEME_CENTRAL4)
    got = _gpu([(spec, q)], 3.385e-3, stages=3)[0]
    ob = _oracle([(spec, q)], 3.385e-3, stages=3)
    errs = state_errors(spec, got, ob.q[0])
    assert max(errs) < 1e-12, errs


def test_curvilinear_four_blocks_full_size_three_stages(built_lib, oracle_lib):
    blocks = problems.curvilinear_multiblock_3d(seed=0)
    assert sum(b[0].npoints for b in blocks) == 12582912
    dt = problems.multiblock_cfl_dt(blocks, 0.5)
    got = _gpu(blocks, dt, stages=3)
    ob = _oracle(blocks, dt, stages=3)
    for b, blk in enumerate(blocks):
        errs = state_errors(blk[0], got[b], ob.q[b])
        assert max(errs) < 1e-12, (b, errs)


def test_persistent_stage_each_ensemble_size_against_oracle(built_lib, oracle_lib):
    """One instance of every size of the KH ensemble, in one persistent batch, FP32 residual,
    one RK step against the FP64 oracle: within the FP32-residual tolerance (1e-6 of the field
    scale after one step of the ensemble's time step)."""
    blocks = [problems.kh(n=n, amp=1.0, phase=0.3 * i) for i, n in enumerate(problems.KH_SIZES)]
    dt = 2e-4
    sched = {"mode": abi.SCHED_PERSISTENT, "tile_y": 16, "ctas_per_sm": 2, "dynamic": 1, "order": 0}
    got = _gpu(blocks, dt, steps=1, precision="fp32", schedule=sched)
    ob = _oracle(blocks, dt, steps=1)
    for b, (spec, _) in enumerate(blocks):
        errs = state_errors(spec, got[b], ob.q[b])
        assert max(errs) < 1e-6, (spec.size, errs)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("fp32", 3e-5)])
def test_curvilinear_3d_teno5_matches_reference_solver(built_lib, precision, tol):
    """The 3D curvilinear TENO5 block (the 4-block configuration's discretisation) on the GPU
    against the reference's own generated solver, from the same state (1e-3 random perturbation)
    with the solver's own metric arrays, per variable on its scale (momenta on the momentum
    scale): 1e-12 in FP64 after 1, 3 and 30 stages; the FP32 residual within 3e-5 (TENO's
    cut-off decisions on the noisy state differ in FP32; its departure after 30 stages is of
    order 1e-5)."""
    from test_oracle_golden import CURV3D, load_case
    from opensbli_gb300.solver import Solver
    blk, _, _, g = load_case(CURV3D)
    spec = blk[0]
    sl = spec.interior()
    dt = float(g["dt"])
    for n in g["counts"]:
        n = int(n)
        nsteps, rest = divmod(n, 3)
        s = Solver([blk], precision=precision, rk="ls3")
        s.apply_bc()
        if nsteps:
            s.step(dt, nsteps)
        for st in range(rest):
            s.stage(st, dt)
        got = s.state(0)
        s.close()
        ref = np.zeros_like(np.stack(got))
        ref[(slice(None),) + sl] = g["after_%d" % n]
        errs = state_errors(spec, got, ref)
        assert max(errs) < tol, (n, errs)
