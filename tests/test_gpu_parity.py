"""GPU parity: the CUDA path (through the C ABI) against the C oracle on seeded inputs.

FP64 tolerances: 1e-12 relative (max |diff| / max |field|) for the well-conditioned schemes
(WENO5-JS, TENO5, central); WENO5-Z is compared on perturbed inputs (its epsilon of 1e-40
amplifies rounding-level differences on flat data -- the reference itself moves by 1e-3
under 1e-15 input noise).  FP32-residual tolerances are stated per test.
"""
import numpy as np
import pytest

import harness
from opensbli_gb300 import abi, problems

pytestmark = pytest.mark.gpu


def _solver(*a, **k):
    from opensbli_gb300.solver import Solver
    return Solver(*a, **k)


def _perturb(q, amp, seed):
    rng = np.random.default_rng(seed)
    return [a * (1.0 + amp * rng.standard_normal(a.shape)) for a in q]


def _run_pair(spec, q, rk, dt, nstages, precision="fp64"):
    kind, A, B = (abi.RK_LOW_STORAGE, problems.RK3_LS_A, problems.RK3_LS_B) if rk == "ls3" else \
        (abi.RK_SBLI3, problems.RK3_SBLI_NEW, problems.RK3_SBLI_OLD)
    s = _solver([(spec, q)], precision=precision, rk=rk)
    s.apply_bc()
    ob = harness.OracleBlocks([(spec, q)])
    ob.apply_bc()
    nsteps, rest = divmod(nstages, 3)
    if nsteps:
        s.step(dt, nsteps)
        ob.step(kind, A, B, dt, nsteps)
    if rest:
        if kind == abi.RK_SBLI3:
            s.save_sbli()
            for v in range(spec.nvars):
                ob.rk[0][v][...] = ob.q[0][v]
        for st in range(rest):
            s.stage(st, dt)
            ob.stage(kind, A, B, st, dt)
    got = s.state(0)
    s.close()
    return state_errors(spec, got, ob.q[0]), got, ob


def state_errors(spec, got, ref):
    """max|diff| per variable, relative to the scale of that quantity: rho and rhoE to their own
    maxima, every momentum component to the largest momentum magnitude (a component may start
    at exactly zero, e.g. w in the TGV)."""
    sl = spec.interior()
    mscale = max(float(np.max(np.abs(ref[1 + i][sl]))) for i in range(spec.ndim))
    out = []
    for v in range(spec.nvars):
        d = float(np.max(np.abs(got[v][sl] - ref[v][sl])))
        scale = mscale if 1 <= v <= spec.ndim else float(np.max(np.abs(ref[v][sl])))
        out.append(d / max(scale, 1e-300))
    return out


@pytest.mark.parametrize("nstages", [1, 3, 30])
def test_sod_weno5js_fp64(built_lib, oracle_lib, nstages):
    spec, q = problems.sod(400)
    errs, _, _ = _run_pair(spec, q, "ls3", 2e-4, nstages)
    assert max(errs) < 1e-12, errs


def test_sod_1000_steps_fp64(built_lib, oracle_lib):
    spec, q = problems.sod(400)
    errs, got, _ = _run_pair(spec, q, "ls3", 2e-4, 3000)
    assert max(errs) < 1e-11, errs


@pytest.mark.parametrize("nstages", [1, 3, 9])
def test_tgv_teno5_fp64(built_lib, oracle_lib, nstages):
    spec, q = problems.tgv(16, minf=1.25, scheme=abi.SCHEME_TENO5, averaging=abi.AVG_ROE)
    errs, _, _ = _run_pair(spec, q, "ls3", 1e-3, nstages)
    assert max(errs) < 1e-12, errs


@pytest.mark.parametrize("nstages", [1, 3])
def test_tgv_weno5z_fp64_perturbed(built_lib, oracle_lib, nstages):
    spec, q = problems.tgv(16, minf=1.25, scheme=abi.SCHEME_WENO5_Z, averaging=abi.AVG_SIMPLE)
    q = _perturb(q, 1e-3, 1)
    errs, _, _ = _run_pair(spec, q, "ls3", 1e-3, nstages)
    assert max(errs) < 1e-11, errs


@pytest.mark.parametrize("nstages", [1, 3, 9])
def test_tgv_central_fp64(built_lib, oracle_lib, nstages):
    spec, q = problems.tgv(16, minf=0.1, scheme=abi.SCHEME_CENTRAL4)
    errs, _, _ = _run_pair(spec, q, "ls3", 3.385e-3, nstages)
    assert max(errs) < 1e-12, errs


def test_tgv_central_anisotropic_fp64(built_lib, oracle_lib):
    spec, q = problems.tgv(minf=0.1, scheme=abi.SCHEME_CENTRAL4, sizes=(40, 12, 20))
    errs, _, _ = _run_pair(spec, q, "ls3", 1e-3, 3)
    assert max(errs) < 1e-12, errs


def test_tgv_teno5_anisotropic_fp64(built_lib, oracle_lib):
    spec, q = problems.tgv(minf=1.25, scheme=abi.SCHEME_TENO5, averaging=abi.AVG_ROE, sizes=(44, 12, 20))
    errs, _, _ = _run_pair(spec, q, "ls3", 1e-3, 3)
    assert max(errs) < 1e-12, errs


@pytest.mark.parametrize("nstages", [1, 3, 6])
def test_kh_weno5z_sbli3_fp64_perturbed(built_lib, oracle_lib, nstages):
    spec, q = problems.kh(32, amp=1.0, phase=0.3)
    q = _perturb(q, 1e-3, 2)
    errs, _, _ = _run_pair(spec, q, "sbli3", 2e-4, nstages)
    assert max(errs) < 1e-10, errs


def test_kh_teno5_roe_fp64_perturbed(built_lib, oracle_lib):
    # the unperturbed KH state is piecewise constant, where TENO's cut-off acts on
    # rounding-level smoothness indicators; compare on a perturbed state
    spec, q = problems.kh(sizes=(40, 24), amp=1.0, scheme=abi.SCHEME_TENO5, averaging=abi.AVG_ROE)
    q = _perturb(q, 1e-3, 3)
    errs, _, _ = _run_pair(spec, q, "ls3", 2e-4, 6)
    assert max(errs) < 1e-12, errs


def test_residual_hook_matches_oracle(built_lib, oracle_lib):
    spec, q = problems.tgv(16, minf=1.25, scheme=abi.SCHEME_TENO5, averaging=abi.AVG_ROE)
    s = _solver([(spec, q)], precision="fp64")
    s.apply_bc()
    R = s.residual(0)
    ob = harness.OracleBlocks([(spec, q)])
    ob.apply_bc()
    Ro = ob.residual(0)
    sl = spec.interior()
    errs = [harness.rel_err(R[v][sl], Ro[v][sl]) for v in range(spec.nvars)]
    s.close()
    assert max(errs) < 1e-12, errs


@pytest.mark.parametrize("what", [abi.RED_KE, abi.RED_RHO_SUM, abi.RED_ENSTROPHY_DISS, abi.RED_DILATATION_DISS,
                                  abi.RED_CFL_DT, abi.RED_NAN_COUNT])
def test_reductions(built_lib, oracle_lib, what):
    spec, q = problems.tgv(16, minf=1.25, scheme=abi.SCHEME_TENO5, averaging=abi.AVG_ROE)
    s = _solver([(spec, q)], precision="fp64")
    s.apply_bc()
    got = s.reduce(what)
    s.close()
    ob = harness.OracleBlocks([(spec, q)])
    ob.apply_bc()
    ref = ob.reduce(what)
    assert abs(got - ref) <= 1e-12 * max(abs(ref), 1.0), (got, ref)


# ---- FP32 residual path ---------------------------------------------------------------

def test_fp32_residual_tgv_teno5_one_step(built_lib, oracle_lib):
    spec, q = problems.tgv(24, minf=1.25, scheme=abi.SCHEME_TENO5, averaging=abi.AVG_ROE)
    errs, _, _ = _run_pair(spec, q, "ls3", 1e-3, 3, precision="fp32")
    assert max(errs) < 1e-6, errs


def test_fp32_residual_sod(built_lib, oracle_lib):
    spec, q = problems.sod(400)
    errs, _, _ = _run_pair(spec, q, "ls3", 2e-4, 300, precision="fp32")
    assert max(errs) < 1e-4, errs


def test_fp32_residual_central(built_lib, oracle_lib):
    spec, q = problems.tgv(16, minf=0.1, scheme=abi.SCHEME_CENTRAL4)
    errs, _, _ = _run_pair(spec, q, "ls3", 3.385e-3, 30, precision="fp32")
    assert max(errs) < 1e-6, errs
