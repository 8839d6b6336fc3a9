"""GPU parity of the Central4-WENO5 benchmark path: the KGP split convective terms
(split_forms.py:178-236) and the non-linear characteristic WENO3 filter with its Ducros sensor
(filters/WENO_filter.py), through the C ABI, against the oracle and against the golden states
of the reference's shipped Central4-WENO5 solver (tests/golden/shipped_c4w5_16.npz)."""
import os

import numpy as np
import pytest

import harness
from opensbli_gb300 import abi, problems

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def c4w5(n=16, sizes=None):
    spec, q = problems.tgv(n, minf=1.25, scheme=abi.SCHEME_CENTRAL4, viscous=abi.VISC_SUTHERLAND, sizes=sizes)
    spec.split_form = abi.SPLIT_KGP
    spec.filter = abi.FILTER_WENO3
    spec.ducros_check = 0.05
    spec.ducros_select = 0.05
    return spec, q


def _solver(*a, **k):
    from opensbli_gb300.solver import Solver
    return Solver(*a, **k)


def test_kgp_residual_matches_oracle(built_lib, oracle_lib):
    """Residual hook (KGP convective + Sutherland viscous terms) on an anisotropic box, FP64,
    1e-12 of each field's scale."""
    spec, q = c4w5(sizes=(18, 16, 14))
    s = _solver([(spec, q)], precision="fp64", rk="ls3")
    s.apply_bc()
    R = s.residual(0)
    s.close()
    ob = harness.OracleBlocks([(spec, q)])
    ob.apply_bc()
    Ro = ob.residual(0)
    sl = spec.interior()
    errs = [harness.rel_err(R[v][sl], Ro[v][sl]) for v in range(5)]
    assert max(errs) < 1e-12, errs


@pytest.mark.parametrize("steps", [1, 2, 5])
def test_filtered_steps_match_shipped_benchmark_fp64(built_lib, steps):
    """Whole filtered steps on the GPU against the reference's shipped Central4-WENO5 solver
    (16^3, the benchmark's own dt), FP64: 1e-10 of each field's scale (rhou2 starts at zero)."""
    g = np.load(os.path.join(GOLD, "shipped_c4w5_16.npz"))
    spec, q = c4w5(16)
    s = _solver([(spec, q)], precision="fp64", rk="ls3")
    s.apply_bc()
    s.step(float(g["dt"]), steps)
    got = s.state(0)
    s.close()
    sl = spec.interior()
    ref = g["after_%d" % steps]
    errs = [harness.rel_err(got[v][sl], ref[v]) for v in range(5)]
    assert max(errs) < 1e-10, errs


def test_filtered_steps_match_oracle_anisotropic_fp64(built_lib, oracle_lib):
    """A non-cubic filtered block (interfaces -1..N-1 and the filter's shifted halo range along
    each extent), 3 steps, FP64 against the oracle: 1e-10."""
    spec, q = c4w5(sizes=(18, 16, 14))
    dt = 0.01
    s = _solver([(spec, q)], precision="fp64", rk="ls3")
    s.apply_bc()
    s.step(dt, 3)
    got = s.state(0)
    s.close()
    ob = harness.OracleBlocks([(spec, q)])
    ob.apply_bc()
    ob.step(abi.RK_LOW_STORAGE, problems.RK3_LS_A, problems.RK3_LS_B, dt, 3)
    sl = spec.interior()
    errs = [harness.rel_err(got[v][sl], ob.q[0][v][sl]) for v in range(5)]
    assert max(errs) < 1e-10, errs


def test_filtered_steps_fp32_residual(built_lib):
    """FP32-residual path (FP64 state, FP32 KGP / viscous terms and FP32 filter increment)
    against the shipped solver's 5-step state: 5e-5 of the field's scale (the momentum
    components against the momentum scale; rhou2 starts at zero).  The filter's WENO3-Z
    weights and rj sensor are formed from FP32 smoothness indicators, whose cancellation sets
    this level (unfiltered FP32 steps agree to 1e-8)."""
    g = np.load(os.path.join(GOLD, "shipped_c4w5_16.npz"))
    spec, q = c4w5(16)
    s = _solver([(spec, q)], precision="fp32", rk="ls3")
    s.apply_bc()
    s.step(float(g["dt"]), 5)
    got = s.state(0)
    s.close()
    sl = spec.interior()
    ref = g["after_5"]
    mscale = max(float(np.max(np.abs(ref[v]))) for v in (1, 2, 3))
    errs = []
    for v in range(5):
        scale = mscale if v in (1, 2, 3) else float(np.max(np.abs(ref[v])))
        errs.append(float(np.max(np.abs(got[v][sl] - ref[v]))) / scale)
    assert max(errs) < 5e-5, errs


def test_filter_descriptor_checks(built_lib):
    """The filter is rejected outside its implemented path; the single-stage entry point
    without allocations refuses it (the filter follows a whole step)."""
    from opensbli_gb300.solver import Solver
    spec, q = problems.tgv(12, minf=1.25, scheme=abi.SCHEME_TENO5, averaging=abi.AVG_ROE)
    spec.filter = abi.FILTER_WENO3
    with pytest.raises(abi.OSBError):
        Solver([(spec, q)], precision="fp64", rk="ls3")
    spec, q = problems.tgv(12, minf=1.25, scheme=abi.SCHEME_TENO5, averaging=abi.AVG_ROE)
    spec.split_form = abi.SPLIT_KGP
    with pytest.raises(abi.OSBError):
        Solver([(spec, q)], precision="fp64", rk="ls3")


# ---- non-linear TVD filter (filters/TVD_filter.py) ----------------------------------------

def _tvd_golden():
    """The perturbed TGV and the golden states of the reference's generated TVD-filtered solver
    (tests/golden/make_golden.py make_tvd)."""
    g = np.load(os.path.join(GOLD, "tgv_kgp_tvd_12_perturbed.npz"))
    spec, q = problems.tgv_tvd(12, kappa=float(g["kappa"]))
    amp, seed = g["pert"]
    rng = np.random.default_rng(int(seed))
    q = [a * (1.0 + float(amp) * rng.standard_normal(a.shape)) for a in q]
    return spec, q, g


@pytest.mark.parametrize("steps", [1, 2, 4])
def test_tvd_filtered_steps_match_reference_fp64(built_lib, steps):
    """Whole TVD-filtered steps on the GPU (KGP central step, the filter's exchange, the point -2
    velocities of the last stage, the three flux directions, the update) against the
    reference's own generated solver, FP64: 1e-12 of each field's scale.  The filter moves the
    state by about 2e-3 of its scale per step here."""
    spec, q, g = _tvd_golden()
    s = _solver([(spec, q)], precision="fp64", rk="ls3")
    s.apply_bc()
    s.step(float(g["dt"]), steps)
    got = s.state(0)
    s.close()
    sl = spec.interior()
    errs = [harness.rel_err(got[v][sl], g["after_%d" % steps][v]) for v in range(5)]
    assert max(errs) < 1e-12, errs


def test_tvd_filtered_steps_match_oracle_anisotropic_fp64(built_lib, oracle_lib):
    """A non-cubic TVD-filtered block, 3 steps with CUDA graphs, FP64 against the oracle: 1e-12."""
    spec, q = problems.tgv_tvd(sizes=(18, 16, 14), kappa=1.25)
    rng = np.random.default_rng(3)
    q = [a * (1.0 + 1e-2 * rng.standard_normal(a.shape)) for a in q]
    dt = 4e-3
    s = _solver([(spec, q)], precision="fp64", rk="ls3")
    s.apply_bc()
    s.step(dt, 3)
    got = s.state(0)
    s.close()
    ob = harness.OracleBlocks([(spec, q)])
    ob.apply_bc()
    ob.step(abi.RK_LOW_STORAGE, problems.RK3_LS_A, problems.RK3_LS_B, dt, 3)
    sl = spec.interior()
    errs = [harness.rel_err(got[v][sl], ob.q[0][v][sl]) for v in range(5)]
    assert max(errs) < 1e-12, errs


def test_tvd_filtered_steps_fp32_residual(built_lib):
    """FP32-residual path (FP32 central terms, FP32 TVD filter increment added to the FP64
    state) against the reference's 4-step state: 1e-5 of each field's scale (the momentum
    components against the momentum scale), 200x below the filter's own effect."""
    spec, q, g = _tvd_golden()
    s = _solver([(spec, q)], precision="fp32", rk="ls3")
    s.apply_bc()
    s.step(float(g["dt"]), 4)
    got = s.state(0)
    s.close()
    sl = spec.interior()
    ref = g["after_4"]
    mscale = max(float(np.max(np.abs(ref[v]))) for v in (1, 2, 3))
    errs = []
    for v in range(5):
        scale = mscale if v in (1, 2, 3) else float(np.max(np.abs(ref[v])))
        errs.append(float(np.max(np.abs(got[v][sl] - ref[v]))) / scale)
    assert max(errs) < 1e-5, errs


def test_tvd_descriptor_checks(built_lib):
    """The TVD filter is refused outside its path: a shock-capturing block, a stage exchange
    shallower than the point -2 it reads, a non-finite kappa_TVD."""
    spec, q = problems.tgv(12, minf=1.25, scheme=abi.SCHEME_TENO5, averaging=abi.AVG_ROE)
    spec.filter = abi.FILTER_TVD
    with pytest.raises(abi.OSBError):
        _solver([(spec, q)], precision="fp64", rk="ls3")
    spec, q = problems.tgv_tvd(12)
    spec.bc_depth = [[1, 1] for _ in range(3)]
    with pytest.raises(abi.OSBError):
        _solver([(spec, q)], precision="fp64", rk="ls3")
    spec, q = problems.tgv_tvd(12, kappa=float("nan"))
    with pytest.raises(abi.OSBError):
        _solver([(spec, q)], precision="fp64", rk="ls3")
