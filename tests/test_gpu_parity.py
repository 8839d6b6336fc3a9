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


@pytest.mark.parametrize("nstages", [1, 3, 30])
def test_sod_extrapolation_fp64(built_lib, oracle_lib, nstages):
    """Linear extrapolation on the left, zeroth order on the right, perturbed state."""
    spec, q = problems.sod(200, bc=(abi.BC_EXTRAP1, abi.BC_EXTRAP0))
    errs, _, _ = _run_pair(spec, _perturb(q, 1e-2, 13), "ls3", 2e-4, nstages)
    assert max(errs) < 1e-12, errs


def test_sod_1000_steps_fp64(built_lib, oracle_lib):
    spec, q = problems.sod(400)
    errs, got, _ = _run_pair(spec, q, "ls3", 2e-4, 3000)
    assert max(errs) < 1e-11, errs


@pytest.mark.parametrize("nstages", [1, 3, 9])
def test_tgv_teno6_fp64(built_lib, oracle_lib, nstages):
    spec, q = problems.tgv(16, minf=1.25, scheme=abi.SCHEME_TENO6, averaging=abi.AVG_ROE)
    errs, _, _ = _run_pair(spec, q, "ls3", 1e-3, nstages)
    assert max(errs) < 1e-12, errs


def _benchmark_reductions(spec, q_last_stage, rho_final):
    """The reference benchmark's post-processing sums (apps/performance_benchmark/TENO6/
    opensbli.cpp:435-457 with its kernel 048): velocities, viscosity and their 4th-order
    derivatives come from the constituent-relation arrays of the last RK stage (the state at
    the start of that stage, halos exchanged), density from the final state."""
    g, minf = spec.gama, spec.Minf
    rho_s = q_last_stage[0]
    u = [q_last_stage[1 + i] / rho_s for i in range(3)]
    p = (g - 1.0) * (q_last_stage[4] - 0.5 * rho_s * (u[0] ** 2 + u[1] ** 2 + u[2] ** 2))
    T = minf * minf * g * p / rho_s
    mu = 1.4042 * T * np.sqrt(T) / (0.40417 + T)
    h = spec.halo
    n = spec.size

    def d1(f, axis, d):
        inv = 1.0 / spec.delta[d]
        return ((-(2.0 / 3.0)) * np.roll(f, 1, axis) - (1.0 / 12.0) * np.roll(f, -2, axis)
                + (1.0 / 12.0) * np.roll(f, 2, axis) + (2.0 / 3.0) * np.roll(f, -1, axis)) * inv
    # arrays are (z, y, x); the interior is away from the wrap of np.roll by the 5 halo layers
    du = [[d1(u[i], 2 - d, d) for d in range(3)] for i in range(3)]
    sl = spec.interior()
    wx = du[2][1] - du[1][2]
    wy = du[0][2] - du[2][0]
    wz = du[1][0] - du[0][1]
    div = du[0][0] + du[1][1] + du[2][2]
    return {"KE": float(np.sum((0.5 * (u[0] ** 2 + u[1] ** 2 + u[2] ** 2) * rho_final)[sl])),
            "dilatation": float(np.sum(((4.0 / 3.0) * div * div * mu)[sl])),
            "enstrophy": float(np.sum(((wx * wx + wy * wy + wz * wz) * mu)[sl])),
            "rhom": float(np.sum(rho_final[sl]))}


def test_teno6_benchmark_known_answer(built_lib):
    """The reference's TENO6 performance benchmark validation (apps/performance_benchmark/
    README.MD, "va" mode): supersonic TGV, 128^3, M=1.25, Re=1600, TENO6 with Roe averaging +
    central-4 viscous terms, RK-LS3, 500 steps of dt = 2 x 0.00084625, printed to 6 digits:
    KE 2.65363e+05, dilatation dissipation 1.16991e+05, enstrophy dissipation 1.79666e+06,
    rhom 2.09715e+06 -- evaluated as that benchmark does (velocities and viscosity of the last
    RK stage, final density)."""
    from opensbli_gb300.solver import Solver
    spec, q = problems.tgv(128, minf=1.25, scheme=abi.SCHEME_TENO6, averaging=abi.AVG_ROE)
    dt = 2 * 0.00084625
    s = Solver([(spec, q)], precision="fp64", rk="ls3")
    s.apply_bc()
    s.step(dt, 499)
    s.stage(0, dt)
    s.stage(1, dt)
    q_last = s.state(0)
    s.stage(2, dt)
    rho_final = s.state(0)[0]
    s.close()
    got = _benchmark_reductions(spec, q_last, rho_final)
    want = {"KE": 2.65363e+05, "dilatation": 1.16991e+05, "enstrophy": 1.79666e+06, "rhom": 2.09715e+06}
    for k in want:
        # the printed value is the exact result rounded to 6 significant digits
        half_ulp = 0.5 * 10.0 ** (np.floor(np.log10(abs(want[k]))) - 5)
        assert abs(got[k] - want[k]) <= half_ulp * (1 + 1e-9), (k, got[k], want[k])


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


@pytest.mark.parametrize("what", [abi.RED_KE, abi.RED_ENSTROPHY_DISS, abi.RED_DILATATION_DISS, abi.RED_CFL_DT])
def test_reductions_stretched_grid(built_lib, oracle_lib, what):
    """Reductions on the stretched wall-normal grid: the y derivatives and the CFL's y term take
    D11 of the row."""
    spec, q = problems.channel_iso((16, 17, 8), stretch=1.7)
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
