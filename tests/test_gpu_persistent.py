"""The persistent fused stage (one launch per RK stage over a batch of 2D periodic blocks,
FP32 residual) against the per-block FP32 path, across its schedules, and the autotuner.

Per-block vs persistent: the same interface fluxes and float-float residual, so the states
agree to FP64 rounding of the RK update (1e-14 relative); the persistent stage's schedules
(tile height, CTAs per SM, tile claiming and order) give bit-identical states.
"""
import numpy as np
import pytest

from opensbli_gb300 import abi, problems

from test_gpu_parity import state_errors

pytestmark = pytest.mark.gpu


def _ensemble(count=3, seed=5, sizes=(64, 96, 128), rng_pert=1e-3):
    blocks = problems.kh_ensemble(count, seed=seed, sizes=sizes)
    rng = np.random.default_rng(seed)
    out = []
    for spec, q in blocks:
        out.append((spec, [a * (1.0 + rng_pert * rng.standard_normal(a.shape)) for a in q]))
    return out


def _run(blocks, sched, nsteps=3, rk="ls3", dt=2e-4, graphs=True):
    from opensbli_gb300.solver import Solver
    s = Solver(blocks, precision="fp32", rk=rk, graphs=graphs)
    s.set_schedule(**sched)
    s.apply_bc()
    s.step(dt, nsteps)
    mode = s.schedule()[0]
    out = [s.state(i) for i in range(len(blocks))]
    s.close()
    return mode, out


PER_BLOCK = {"mode": abi.SCHED_PER_BLOCK}
PERSIST = {"mode": abi.SCHED_PERSISTENT, "tile_y": 16, "ctas_per_sm": 2, "dynamic": 1, "order": 0}


@pytest.mark.parametrize("rk", ["ls3", "sbli3"])
def test_persistent_matches_per_block(built_lib, rk):
    blocks = _ensemble()
    m0, a = _run(blocks, PER_BLOCK, rk=rk)
    m1, b = _run(blocks, PERSIST, rk=rk)
    assert (m0, m1) == (abi.SCHED_PER_BLOCK, abi.SCHED_PERSISTENT)
    for i, (spec, _) in enumerate(blocks):
        errs = state_errors(spec, b[i], a[i])
        assert max(errs) < 1e-14, (i, errs)
        # halos refreshed at the end of the step (periodic images, depth 4)
        h = spec.halo
        n0, n1 = spec.size[0], spec.size[1]
        assert np.array_equal(b[i][0][h:h + n1, 1:h], b[i][0][h:h + n1, n0 + 1:n0 + h])


@pytest.mark.parametrize("ty,cps,dyn,order", [(8, 1, 0, 0), (32, 3, 1, 1), (16, 4, 0, 2), (8, 2, 1, 2)])
def test_persistent_schedules_are_bit_identical(built_lib, ty, cps, dyn, order):
    blocks = _ensemble(count=4, seed=6, sizes=(64, 96))
    _, ref = _run(blocks, PERSIST, nsteps=2)
    _, got = _run(blocks, {"mode": abi.SCHED_PERSISTENT, "tile_y": ty, "ctas_per_sm": cps, "dynamic": dyn,
                           "order": order}, nsteps=2)
    for i in range(len(blocks)):
        for v in range(4):
            assert np.array_equal(got[i][v], ref[i][v]), (i, v)


def test_persistent_without_graphs_and_odd_step_counts(built_lib):
    """Eager launches and graph replays over both FP32-buffer parities give the same states."""
    blocks = _ensemble(count=2, seed=7, sizes=(64,))
    _, a = _run(blocks, PERSIST, nsteps=5, graphs=False)
    _, b = _run(blocks, PERSIST, nsteps=5, graphs=True)
    for i in range(len(blocks)):
        for v in range(4):
            assert np.array_equal(a[i][v], b[i][v]), (i, v)


def test_persistent_stage_hook_and_residual(built_lib):
    """osb_stage in the persistent schedule matches osb_step's stages; osb_residual still
    reads the current FP32 state."""
    from opensbli_gb300.solver import Solver
    blocks = _ensemble(count=2, seed=8, sizes=(64,))
    s = Solver(blocks, precision="fp32", rk="ls3")
    s.set_schedule(**PERSIST)
    s.apply_bc()
    for st in range(3):
        s.stage(st, 2e-4)
    staged = [s.state(i) for i in range(2)]
    r = s.residual(0)
    s.close()
    _, stepped = _run(blocks, PERSIST, nsteps=1)
    for i in range(2):
        for v in range(4):
            assert np.array_equal(staged[i][v], stepped[i][v]), (i, v)
    assert all(np.isfinite(x).all() for x in r)


def test_persistent_rejected_where_ineligible(built_lib):
    from opensbli_gb300.solver import Solver
    spec, q = problems.tgv(12, minf=1.25, scheme=abi.SCHEME_TENO5, averaging=abi.AVG_ROE)
    s = Solver([(spec, q)], precision="fp32")
    with pytest.raises(abi.OSBError) as e:
        s.set_schedule(**PERSIST)
    assert "2D" in str(e.value)
    assert s.schedule()[0] == abi.SCHED_PER_BLOCK
    s.close()


def test_autotune_picks_and_caches(built_lib, tmp_path):
    from opensbli_gb300 import autotune
    from opensbli_gb300.solver import Solver
    blocks = _ensemble(count=3, seed=9, sizes=(64, 128))
    cache = str(tmp_path / "tune.json")
    s = Solver(blocks, precision="fp32")
    s.apply_bc()
    before = [s.state(i) for i in range(3)]
    cands = autotune.candidates(True)[:5]
    best, trials = autotune.tune(s, 2e-4, steps=2, warmup=1, cache=cache, cands=cands)
    assert len(trials) == 5 and best in cands
    after = [s.state(i) for i in range(3)]
    for i in range(3):
        for v in range(4):
            assert np.array_equal(before[i][v], after[i][v])  # the trials left no trace
    s.close()
    s = Solver(blocks, precision="fp32")
    best2, trials2 = autotune.tune(s, 2e-4, cache=cache)
    assert best2 == best and trials2 == []
    s.close()
