"""GPU parity of curvilinear blocks and block interfaces: the CUDA path (through the C ABI)
against the C oracle, plus the reference's own curvilinear known answer.

FP64 tolerance 1e-12 relative (max |diff| / field scale, momentum against the momentum
scale); the FP32-residual tolerance is stated per test.
"""
import numpy as np
import pytest

import harness
from opensbli_gb300 import abi, problems

from test_gpu_parity import state_errors

pytestmark = pytest.mark.gpu

LS = (abi.RK_LOW_STORAGE, problems.RK3_LS_A, problems.RK3_LS_B)


def _solver(*a, **k):
    from opensbli_gb300.solver import Solver
    return Solver(*a, **k)


def _run_blocks(blocks, dt, nsteps, precision="fp64", stages=0):
    s = _solver(blocks, precision=precision, rk="ls3")
    s.apply_bc()
    if nsteps:
        s.step(dt, nsteps)
    for st in range(stages):
        s.stage(st, dt)
    got = [s.state(i) for i in range(len(blocks))]
    s.close()
    return got


def _oracle_blocks(blocks, dt, nsteps, stages=0):
    ob = harness.OracleBlocks(blocks)
    ob.apply_bc()
    if nsteps:
        ob.step(*LS, dt, nsteps)
    for st in range(stages):
        ob.stage(*LS, st, dt)
    return ob


@pytest.mark.parametrize("nsteps,stages", [(0, 1), (1, 0), (5, 0)])
def test_curvilinear_2d_fp64(built_lib, oracle_lib, nsteps, stages):
    blk = problems.curvilinear_wave_2d(32)
    got = _run_blocks([blk], 5e-4, nsteps, stages=stages)[0]
    ob = _oracle_blocks([blk], 5e-4, nsteps, stages)
    errs = state_errors(blk[0], got, ob.q[0])
    assert max(errs) < 1e-12, errs


def test_curvilinear_known_answer_gpu(built_lib):
    """The reference's known answer (tests/verification_apps/euler_wave_curvilinear): rho at
    index [69, 69] of the halo-inclusive array after 10 steps on 128^2 is 0.9984292346559068
    to 1e-9 relative."""
    blk = problems.curvilinear_wave_2d(128)
    got = _run_blocks([blk], 5e-4, 10)[0]
    rho = got[0][69, 69]
    assert abs(rho - 0.9984292346559068) < 1e-9 * 0.9984292346559068, rho


SMALL = {"A": (32, 16, 8), "B": (16, 16, 8), "C": (32, 8, 8), "D": (16, 16, 8)}


@pytest.mark.parametrize("nsteps", [1, 3])
def test_curvilinear_multiblock_3d_fp64(built_lib, oracle_lib, nsteps):
    blocks = problems.curvilinear_multiblock_3d(sizes=SMALL, seed=1)
    dt = problems.multiblock_cfl_dt(blocks, 0.5)
    got = _run_blocks(blocks, dt, nsteps)
    ob = _oracle_blocks(blocks, dt, nsteps)
    for b, (spec, _, _) in enumerate(blocks):
        errs = state_errors(spec, got[b], ob.q[b])
        assert max(errs) < 1e-12, (b, errs)


def test_split_block_equals_single_block(built_lib, oracle_lib):
    """A periodic block cut into three pieces joined by interfaces advances exactly like the
    uncut block (viscous TGV: the central terms read the interface corners)."""
    rng = np.random.default_rng(3)
    spec, q = problems.tgv(minf=1.25, scheme=abi.SCHEME_TENO5, averaging=abi.AVG_ROE,
                           viscous=abi.VISC_SUTHERLAND, sizes=(20, 12, 12))
    q = [a * (1.0 + 1e-3 * rng.standard_normal(a.shape)) for a in q]
    parts = problems.split_block(spec, q, [8, 14], d=0)
    one = _run_blocks([(spec, q)], 1e-3, 2)[0]
    many = _run_blocks(parts, 1e-3, 2)
    ob = _oracle_blocks(parts, 1e-3, 2)
    edges = [0, 8, 14, 20]
    sl = spec.interior()
    for b, (ps, _) in enumerate(parts):
        for v in range(spec.nvars):
            ref = one[v][sl][:, :, edges[b]:edges[b + 1]]
            assert np.array_equal(many[b][v][ps.interior()], ref), (b, v)
        errs = state_errors(ps, many[b], ob.q[b])
        assert max(errs) < 1e-12, (b, errs)


def test_split_curvilinear_2d_along_y(built_lib, oracle_lib):
    """Interfaces normal to y on a curvilinear block: the pieces match the uncut block."""
    spec, q, met = problems.curvilinear_wave_2d(32)
    parts = problems.split_block(spec, q, [12], d=1, metrics=met)
    one = _run_blocks([(spec, q, met)], 5e-4, 3)[0]
    many = _run_blocks(parts, 5e-4, 3)
    sl = spec.interior()
    edges = [0, 12, 32]
    for b, (ps, _, _) in enumerate(parts):
        for v in range(spec.nvars):
            ref = one[v][sl][edges[b]:edges[b + 1], :]
            assert np.array_equal(many[b][v][ps.interior()], ref), (b, v)


@pytest.mark.parametrize("scheme,tol", [(abi.SCHEME_WENO5_JS, 1e-6), (abi.SCHEME_TENO5, 2e-5)])
def test_fp32_residual_curvilinear_multiblock(built_lib, scheme, tol):
    """FP32-residual path against the FP64 path on the 4-block curvilinear case (8 points per
    wavelength of the mesh in z), 3 steps.  WENO5-JS (smooth weights) stays at the FP32
    rounding level of the residual (measured 2.6e-7); TENO5 is looser (measured 6.9e-6)
    because its binary cut-off picks a different candidate stencil at a few points where the
    FP32 and FP64 smoothness ratios straddle C_T on this under-resolved mesh."""
    blocks = problems.curvilinear_multiblock_3d(sizes=SMALL, seed=2, scheme=scheme)
    dt = problems.multiblock_cfl_dt(blocks, 0.5)
    g64 = _run_blocks(blocks, dt, 3, precision="fp64")
    g32 = _run_blocks(blocks, dt, 3, precision="fp32")
    for b, (spec, _, _) in enumerate(blocks):
        errs = state_errors(spec, g32[b], g64[b])
        assert max(errs) < tol, (b, errs)


def test_fp32_residual_curvilinear_2d(built_lib):
    """FP32-residual path on the resolved 2D curvilinear wave: below 1e-7 after 3 steps
    (measured 2.9e-8)."""
    blk = problems.curvilinear_wave_2d(64)
    g64 = _run_blocks([blk], 5e-4, 3, precision="fp64")[0]
    g32 = _run_blocks([blk], 5e-4, 3, precision="fp32")[0]
    errs = state_errors(blk[0], g32, g64)
    assert max(errs) < 1e-7, errs


def test_interface_validation(built_lib):
    """An interface naming a missing block or a face of another size is rejected with
    OSB_EINVAL before any kernel runs."""
    spec, q = problems.tgv(minf=1.25, scheme=abi.SCHEME_TENO5, averaging=abi.AVG_ROE, sizes=(12, 12, 12))
    parts = problems.split_block(spec, q, [6], d=0)
    bad = parts[0][0]
    bad.iface[0][0] = (7, 0, 1, 0)
    s = _solver(parts, precision="fp64")
    with pytest.raises(abi.OSBError) as e:
        s.apply_bc()
    assert "names block 7" in str(e.value)
    s.close()


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("fp32", 1e-6)])
def test_flipped_interfaces_match_reference_solver(built_lib, precision, tol):
    """Two blocks joined by flipped interfaces (the InterfaceBC match flag of a C-mesh wake cut:
    the neighbour's layers in reverse order along the normal), periodic in y, on the GPU against
    the reference's generated multi-block solver (golden states after 1, 3 and 30 stages, both
    blocks, from the same perturbed states)."""
    import os
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "mb2_flip_24x20_perturbed.npz"))
    from test_oracle_golden import perturb
    blocks = [(s, perturb(q, float(g["pert"][0]), int(g["pert"][1]))) for s, q in problems.flipped_pair_2d((24, 20))]
    dt = float(g["dt"])
    for n in g["counts"]:
        n = int(n)
        got = _run_blocks(blocks, dt, n // 3, stages=n % 3, precision=precision)
        for b, (spec, _) in enumerate(blocks):
            ref = np.zeros((4,) + spec.shape)
            ref[(slice(None),) + spec.interior()] = g["after_%d_%d" % (n, b)]
            errs = state_errors(spec, got[b], ref)
            assert max(errs) < tol, (n, b, errs)
