"""Checkpoint / restart: a run that writes a restart file after k steps, and a fresh solver
(or backend) that reads it and continues, end bit-identical to the uninterrupted run -- state
and RK register, both precisions, the low-storage and SBLI integrators, the persistent batched
stage and a run driven through GB300Backend."""
import os

import numpy as np
import pytest

from opensbli_gb300 import abi, problems

pytestmark = pytest.mark.gpu


def _straight_and_restarted(blocks, precision, rk, dt, n1, n2, tmp_path, schedule=None):
    from opensbli_gb300.solver import Solver

    def make(items):
        s = Solver(items, precision=precision, rk=rk)
        if schedule is not None:
            s.set_schedule(**schedule)
        return s

    a = make(blocks)
    a.apply_bc()
    a.step(dt, n1 + n2)
    ref = [(a.state(i), a.rk_register(i)) for i in range(len(blocks))]
    a.close()

    b = make(blocks)
    b.apply_bc()
    b.step(dt, n1)
    path = str(tmp_path / "restart.npz")
    b.save_restart(path, n1, n1 * dt)
    b.close()
    # a fresh solver starting from a different state: the file replaces it
    zero = [(blk[0], [np.full(blk[0].shape, 1.0) for _ in range(blk[0].nvars)]) + tuple(blk[2:]) for blk in blocks]
    c = make(zero)
    it, t = c.load_restart(path)
    assert it == n1 and t == n1 * dt
    c.apply_bc()
    c.step(dt, n2)
    got = [(c.state(i), c.rk_register(i)) for i in range(len(blocks))]
    c.close()
    return ref, got


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_restart_is_bit_identical_tgv(built_lib, tmp_path, precision):
    spec, q = problems.tgv(16, minf=1.25, scheme=abi.SCHEME_TENO5, averaging=abi.AVG_ROE)
    ref, got = _straight_and_restarted([(spec, q)], precision, "ls3", 1e-3, 2, 2, tmp_path)
    for (qa, ra), (qb, rb) in zip(ref, got):
        for v in range(spec.nvars):
            assert np.array_equal(qa[v], qb[v]), ("state", v)
            assert np.array_equal(ra[v][spec.interior()], rb[v][spec.interior()]), ("register", v)


def test_restart_is_bit_identical_sbli_persistent(built_lib, tmp_path):
    """Two KH instances on the persistent batched stage, SBLI RK3, FP32 residual."""
    blocks = [problems.kh(48, amp=1.0, phase=0.2), problems.kh(64, amp=0.7, phase=1.0)]
    sched = {"mode": abi.SCHED_PERSISTENT, "tile_y": 16, "ctas_per_sm": 2, "dynamic": 1, "order": 0}
    ref, got = _straight_and_restarted(blocks, "fp32", "sbli3", 2e-4, 3, 2, tmp_path, schedule=sched)
    for b, ((qa, _), (qb, _)) in enumerate(zip(ref, got)):
        spec = blocks[b][0]
        for v in range(spec.nvars):
            assert np.array_equal(qa[v][spec.interior()], qb[v][spec.interior()]), (b, v)


def test_restart_curvilinear_multiblock(built_lib, tmp_path):
    blocks = problems.curvilinear_multiblock_3d(sizes={"A": (32, 16, 8), "B": (16, 16, 8), "C": (32, 8, 8),
                                                       "D": (16, 16, 8)}, seed=2)
    dt = problems.multiblock_cfl_dt(blocks, 0.5)
    ref, got = _straight_and_restarted(blocks, "fp64", "ls3", dt, 2, 1, tmp_path)
    for b, ((qa, _), (qb, _)) in enumerate(zip(ref, got)):
        spec = blocks[b][0]
        for v in range(spec.nvars):
            assert np.array_equal(qa[v][spec.interior()], qb[v][spec.interior()]), (b, v)


def test_backend_restart(built_lib, tmp_path):
    """GB300Backend.save after k steps and initialise(restart=...) continue like the straight
    run, with the iteration count and simulation time restored."""
    from opensbli_gb300.backend import BackendPlan, GB300Backend
    plan = BackendPlan.load(os.path.join(os.path.dirname(__file__), "golden", "plan_shock_64x32.npz"))
    a = GB300Backend.from_plan(plan).initialise().run(6)
    ref = a.state(0)
    a.close()
    b = GB300Backend.from_plan(plan).initialise().run(4)
    path = str(tmp_path / "bk.npz")
    b.save(path)
    b.close()
    c = GB300Backend.from_plan(plan).initialise(restart=path)
    assert c.iteration == 4 and abs(c.simulation_time - 4 * plan.dt) < 1e-15
    c.run(2)
    got = c.state(0)
    assert c.iteration == 6
    c.close()
    for v in range(4):
        assert np.array_equal(ref[v], got[v]), v


def test_restart_refuses_other_blocks(built_lib, tmp_path):
    from opensbli_gb300.solver import Solver
    spec, q = problems.tgv(12, minf=1.25, scheme=abi.SCHEME_TENO5, averaging=abi.AVG_ROE)
    s = Solver([(spec, q)], precision="fp64")
    path = str(tmp_path / "r.npz")
    s.save_restart(path, 0, 0.0)
    s.close()
    spec2, q2 = problems.tgv(14, minf=1.25, scheme=abi.SCHEME_TENO5, averaging=abi.AVG_ROE)
    s2 = Solver([(spec2, q2)], precision="fp64")
    with pytest.raises(ValueError):
        s2.load_restart(path)
    s2.close()
