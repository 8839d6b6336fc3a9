"""Boundary kernels on the GPU against the oracle and against the periodic definition, halos
included: a block whose faces are all periodic gets its whole halo shell in one launch, which
must leave exactly what the direction-by-direction exchange of the reference (ExchangeSelf,
periodic.py:53-71, x then y then z with corners) leaves."""
import numpy as np
import pytest

import harness
from opensbli_gb300 import abi, problems

pytestmark = pytest.mark.gpu


def _scramble(q, seed):
    """Random values everywhere, halos included, so stale halos cannot pass by accident."""
    rng = np.random.default_rng(seed)
    return [1.0 + rng.random(a.shape) for a in q]


def _wrapped(a, spec, depth):
    """The interior of `a` wrapped onto the box [-depth, N + depth) of every used direction."""
    h = spec.halo
    idx = []
    for ax in range(a.ndim):
        d = spec.ndim - 1 - ax  # arrays are (z, y, x)
        n = spec.size[d]
        c = np.arange(-depth, n + depth)
        idx.append(h + np.mod(c, n))
    return a[np.ix_(*idx)]


def _box(a, spec, depth):
    h = spec.halo
    return a[tuple(slice(h - depth, h + spec.size[spec.ndim - 1 - ax] + depth) for ax in range(a.ndim))]


@pytest.mark.parametrize("case", ["3d", "2d", "1d"])
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_periodic_shell_matches_exchange_and_wrap(built_lib, case, precision):
    from opensbli_gb300.solver import Solver
    if case == "3d":
        spec, q = problems.tgv(sizes=(11, 7, 6), scheme=abi.SCHEME_TENO5, averaging=abi.AVG_ROE)
    elif case == "2d":
        spec, q = problems.kh(sizes=(9, 6))
    else:
        spec, q = problems.sod(13, bc=(abi.BC_PERIODIC, abi.BC_PERIODIC))
    depth = spec.bc_depth[0][0]
    q = _scramble(q, 3)
    s = Solver([(spec, q)], precision=precision, rk="ls3")
    s.apply_bc()
    got = s.state(0)
    s.close()
    ob = harness.OracleBlocks([(spec, q)])
    ob.apply_bc()
    ref = ob.q[0]
    for v in range(spec.nvars):
        assert np.array_equal(got[v], ref[v]), (case, v, "oracle")
        assert np.array_equal(_box(got[v], spec, depth), _wrapped(got[v], spec, depth)), (case, v, "wrap")


def _scaled_errors(got, ref, sl):
    """Max error of each field over its scale; the momentum components over the momentum scale
    (rhou1 is zero in the free stream, so its own maximum is set by the top boundary alone)."""
    mscale = max(float(np.max(np.abs(ref[v]))) for v in (1, 2))
    return [float(np.max(np.abs(got[v][sl] - ref[v]))) / (mscale if v in (1, 2) else float(np.max(np.abs(ref[v]))))
            for v in range(4)]


def _shock_case():
    import os
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                             "shock_reflection_64x32_perturbed.npz"))
    spec, q = problems.shock_reflection(64, 32)
    rng = np.random.default_rng(4)
    q = [a * (1.0 + 1e-2 * rng.standard_normal(a.shape)) for a in q]
    return spec, q, g


def test_shock_reflection_boundaries_fp64(built_lib, oracle_lib):
    """Dirichlet inlet and top (the post-shock state from x = 40), extrapolation outlet and
    symmetry wall of the inviscid shock-reflection app, WENO5-Z, 10 steps from a perturbed
    state: against the reference's generated solver (golden, 30 stages) 1e-12 on the interior,
    and against the oracle on every point the boundary kernels and stages write (the whole
    allocation but the corners outside the generated ranges) 1e-12."""
    from opensbli_gb300.solver import Solver
    spec, q, g = _shock_case()
    dt = float(g["dt"])
    s = Solver([(spec, q)], precision="fp64", rk="ls3")
    s.apply_bc()
    s.step(dt, 10)
    got = s.state(0)
    s.close()
    sl = spec.interior()
    errs = [harness.rel_err(got[v][sl], g["after_30"][v]) for v in range(4)]
    assert max(errs) < 1e-12, errs
    ob = harness.OracleBlocks([(spec, q)])
    ob.apply_bc()
    ob.step(abi.RK_LOW_STORAGE, problems.RK3_LS_A, problems.RK3_LS_B, dt, 10)
    h, (n0, n1) = spec.halo, spec.size
    box = (slice(h - 3, h + n1 + 4), slice(h - 3, h + n0 + 4))
    for v in range(4):
        assert np.max(np.abs(got[v][box] - ob.q[0][v][box])) < 1e-12 * np.max(np.abs(ob.q[0][v])), v


def test_shock_reflection_boundaries_fp32(built_lib):
    """The same in the FP32-residual path (FP32 halos from the Dirichlet values and the mirror):
    1e-6 of each field's scale (momentum: the momentum scale) after 10 steps against the
    reference's golden state."""
    from opensbli_gb300.solver import Solver
    spec, q, g = _shock_case()
    s = Solver([(spec, q)], precision="fp32", rk="ls3")
    s.apply_bc()
    s.step(float(g["dt"]), 10)
    got = s.state(0)
    s.close()
    sl = spec.interior()
    errs = _scaled_errors(got, g["after_30"], sl)
    assert max(errs) < 1e-6, errs


def test_dirichlet_needs_values(built_lib):
    from opensbli_gb300.solver import Solver
    spec, q = problems.shock_reflection(40, 20)
    spec.dirichlet = {(0, 0): spec.dirichlet[(0, 0)]}  # the top face has none
    with pytest.raises(abi.OSBError):
        Solver([(spec, q)], precision="fp64", rk="ls3")


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("fp32", 1e-6)])
def test_shock_reflection_ssp_rk3(built_lib, precision, tol):
    """The shock-reflection app's own time integrator, the three-stage SSP coefficients of the
    low-storage form (A = 0 on the first and the last stage), 10 steps against the reference's
    generated solver (golden, 30 stages)."""
    import os
    from opensbli_gb300.solver import Solver
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                             "shock_reflection_ssp_64x32_perturbed.npz"))
    spec, q = problems.shock_reflection(64, 32)
    rng = np.random.default_rng(4)
    q = [a * (1.0 + 1e-2 * rng.standard_normal(a.shape)) for a in q]
    s = Solver([(spec, q)], precision=precision, rk=(abi.RK_LOW_STORAGE, problems.RK3_SSP_A, problems.RK3_SSP_B))
    s.apply_bc()
    s.step(float(g["dt"]), 10)
    got = s.state(0)
    s.close()
    sl = spec.interior()
    errs = _scaled_errors(got, g["after_30"], sl)
    assert max(errs) < tol, errs


def _golden_shock(name, **kw):
    import os
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", name))
    spec, q = problems.shock_reflection(64, 32, **kw)
    rng = np.random.default_rng(4)
    q = [a * (1.0 + 1e-2 * rng.standard_normal(a.shape)) for a in q]
    return spec, q, g


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("fp32", 1e-5)])
def test_hllc_lm_flux_matches_reference_solver(built_lib, oracle_lib, precision, tol):
    """The shock-reflection app with its own HLLC-LM flux (WENO5-Z reconstructed states, simple
    average) and SSP RK3 on the GPU: 10 steps against the reference's generated solver (golden,
    30 stages) and, in FP64, against the oracle on the interior (1e-12)."""
    from opensbli_gb300.solver import Solver
    spec, q, g = _golden_shock("shock_reflection_hllc_64x32_perturbed.npz", flux_type=abi.FLUX_HLLC_LM)
    rk = (abi.RK_LOW_STORAGE, problems.RK3_SSP_A, problems.RK3_SSP_B)
    s = Solver([(spec, q)], precision=precision, rk=rk)
    s.apply_bc()
    s.step(float(g["dt"]), 10)
    got = s.state(0)
    s.close()
    sl = spec.interior()
    errs = _scaled_errors(got, g["after_30"], sl)
    assert max(errs) < tol, errs
    if precision == "fp64":
        ob = harness.OracleBlocks([(spec, q)])
        ob.apply_bc()
        ob.step(*rk, float(g["dt"]), 10)
        errs = [harness.rel_err(got[v][sl], ob.q[0][v][sl]) for v in range(4)]
        assert max(errs) < 1e-12, errs


def test_hllc_lm_residual_matches_oracle_3d(built_lib, oracle_lib):
    """The HLLC-LM sweeps in 3D (the local frames of the y and z sweeps permute the tangential
    momenta): the residual of a perturbed 3D block (the wavy-mesh wave's state on a Cartesian
    grid, every field non-flat) with the HLLC-LM flux and TENO5 against the oracle, FP64, 1e-12
    of each field's scale.  (A state with an exactly zero momentum component, such as the TGV's
    w, makes TENO's cut-off on that wave a decision between rounding-level values.)"""
    from opensbli_gb300.solver import Solver
    spec, q, _, _ = problems.curvilinear_wave_3d((14, 12, 10))
    spec.curvilinear = False
    spec.flux_type = abi.FLUX_HLLC_LM
    rng = np.random.default_rng(8)
    q = [a + 1e-3 * np.max(np.abs(a)) * rng.standard_normal(a.shape) for a in q]
    s = Solver([(spec, q)], precision="fp64", rk="ls3")
    s.apply_bc()
    R = s.residual(0)
    s.close()
    ob = harness.OracleBlocks([(spec, q)])
    ob.apply_bc()
    Ro = ob.residual(0)
    sl = spec.interior()
    scale = max(float(np.max(np.abs(Ro[v][sl]))) for v in range(1, 4))
    for v in range(5):
        sc = scale if 1 <= v <= 3 else float(np.max(np.abs(Ro[v][sl])))
        assert float(np.max(np.abs(R[v][sl] - Ro[v][sl]))) < 1e-12 * sc, v


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("fp32", 1e-6)])
def test_pressure_outlet_matches_reference_solver(built_lib, oracle_lib, precision, tol):
    """PressureOutletBC (back pressure 0.2) in place of the extrapolation outlet: 10 steps
    against the reference's generated solver (golden, 30 stages) and, in FP64, against the
    oracle on the interior and the outlet's plane and halo layers."""
    from opensbli_gb300.solver import Solver
    spec, q, g = _golden_shock("shock_reflection_pout_64x32_perturbed.npz", back_pressure=0.2)
    s = Solver([(spec, q)], precision=precision, rk="ls3")
    s.apply_bc()
    s.step(float(g["dt"]), 10)
    got = s.state(0)
    s.close()
    sl = spec.interior()
    errs = _scaled_errors(got, g["after_30"], sl)
    assert max(errs) < tol, errs
    if precision == "fp64":
        ob = harness.OracleBlocks([(spec, q)])
        ob.apply_bc()
        ob.step(abi.RK_LOW_STORAGE, problems.RK3_LS_A, problems.RK3_LS_B, float(g["dt"]), 10)
        h, (n0, n1) = spec.halo, spec.size
        box = (slice(h, h + n1), slice(h, h + n0 + 4))  # interior rows, through the outlet's 4 halo layers
        for v in range(4):
            assert np.max(np.abs(got[v][box] - ob.q[0][v][box])) < 1e-12 * np.max(np.abs(ob.q[0][v])), v


CHANNELS = {"iso": ("channel_iso_16x17x8_perturbed.npz", "isothermal", 41, None),
            "adi": ("channel_adi_16x17x8_perturbed.npz", "adiabatic", 42, None),
            "str": ("channel_str_16x17x8_perturbed.npz", "isothermal", 43, 1.7)}


def _golden_channel(kind="iso"):
    """The golden channel: isothermal walls on both y faces ("iso"), the upper one adiabatic
    ("adi"), or isothermal walls on the stretched wall-normal grid of the TENO channel app ("str")."""
    import os
    name, upper, seed, stretch = CHANNELS[kind]
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", name))
    spec, q = problems.channel_iso((16, 17, 8), upper=upper, stretch=stretch)
    rng = np.random.default_rng(seed)
    q = [a * (1.0 + 1e-3 * rng.standard_normal(a.shape)) for a in q]
    return spec, q, g


def _channel_errors(got, ref, sl):
    """Max error of each field over its scale, the momentum components over the momentum scale."""
    mscale = max(float(np.max(np.abs(ref[v]))) for v in (1, 2, 3))
    return [float(np.max(np.abs(got[v][sl] - ref[v]))) / (mscale if v in (1, 2, 3) else float(np.max(np.abs(ref[v]))))
            for v in range(5)]


# FP32: the golden state carries 1e-3 relative noise, on which TENO5's binary cut-off decisions
# sit near their threshold, so FP32 rounding flips some of them: 2.6e-5 of the momentum scale
# after 30 stages, the same as the perturbed curvilinear TENO5 case (test_gpu_fullsize.py)
@pytest.mark.parametrize("kind", sorted(CHANNELS))
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("fp32", 5e-5)])
def test_wall_channel_matches_reference_solver(built_lib, oracle_lib, kind, precision, tol):
    """The 3D channel between isothermal no-slip walls (TENO5 + viscous terms with the Carpenter
    closures at both walls) on the GPU: 10 steps against the reference's generated solver
    (golden, 30 stages) and, in FP64, against the oracle on the interior and the walls' halo
    layers (1e-12); with the upper wall adiabatic, and on the stretched wall-normal grid (the y
    flux difference and every y derivative of the viscous terms scaled by D11, SD111 terms)."""
    from opensbli_gb300.solver import Solver
    spec, q, g = _golden_channel(kind)
    s = Solver([(spec, q)], precision=precision, rk="ls3")
    s.apply_bc()
    s.step(float(g["dt"]), 10)
    got = s.state(0)
    s.close()
    sl = spec.interior()
    errs = _channel_errors(got, g["after_30"], sl)
    assert max(errs) < tol, errs
    if precision == "fp64":
        ob = harness.OracleBlocks([(spec, q)])
        ob.apply_bc()
        ob.step(abi.RK_LOW_STORAGE, problems.RK3_LS_A, problems.RK3_LS_B, float(g["dt"]), 10)
        h, (n0, n1, n2) = spec.halo, spec.size
        box = (slice(h, h + n2), slice(h - 4, h + n1 + 4), slice(h, h + n0))  # interior x, z; y through the walls' halos
        for v in range(5):
            assert np.max(np.abs(got[v][box] - ob.q[0][v][box])) < 1e-12 * np.max(np.abs(ob.q[0][v][box])), v


def test_teno_channel_app_matches_reference_solver(built_lib, oracle_lib):
    """The TENO turbulent-channel app's discretisation (TENO6, power-law viscosity mu = T^0.7,
    the constant forcing -c_i / -c_j u_j, isothermal walls on the stretched wall-normal grid, SSP
    RK3), FP64 on the GPU: 10 steps against the reference's generated solver (golden, 30 stages)
    and the oracle, through the walls' halo layers, at 1e-12; the residual of one stage at 1e-12."""
    import os
    from opensbli_gb300.solver import Solver
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "channel_tcf_16x17x8_perturbed.npz"))
    spec, q = problems.channel_tcf((16, 17, 8))
    rng = np.random.default_rng(44)
    q = [a * (1.0 + 1e-3 * rng.standard_normal(a.shape)) for a in q]
    rk = (abi.RK_LOW_STORAGE, problems.RK3_SSP_A, problems.RK3_SSP_B)
    s = Solver([(spec, q)], precision="fp64", rk=rk)
    s.apply_bc()
    R = s.residual(0)
    s.step(float(g["dt"]), 10)
    got = s.state(0)
    s.close()
    sl = spec.interior()
    errs = _channel_errors(got, g["after_30"], sl)
    assert max(errs) < 1e-12, errs
    ob = harness.OracleBlocks([(spec, q)])
    ob.apply_bc()
    Ro = ob.residual(0)
    for v in range(5):
        assert harness.rel_err(R[v][sl], Ro[v][sl]) < 1e-12, ("residual", v)
    ob.step(*rk, float(g["dt"]), 10)
    h, (n0, n1, n2) = spec.halo, spec.size
    box = (slice(h, h + n2), slice(h - 4, h + n1 + 4), slice(h, h + n0))
    for v in range(5):
        assert np.max(np.abs(got[v][box] - ob.q[0][v][box])) < 1e-12 * np.max(np.abs(ob.q[0][v][box])), v


@pytest.mark.parametrize("kind", sorted(CHANNELS))
def test_wall_residual_matches_oracle(built_lib, oracle_lib, kind):
    """The residual of one stage (sweeps plus the viscous terms with the wall closures) of the
    golden channel state, FP64 GPU against the oracle: 1e-12 of each field's scale."""
    from opensbli_gb300.solver import Solver
    spec, q, _ = _golden_channel(kind)
    s = Solver([(spec, q)], precision="fp64", rk="ls3")
    s.apply_bc()
    R = s.residual(0)
    s.close()
    ob = harness.OracleBlocks([(spec, q)])
    ob.apply_bc()
    Ro = ob.residual(0)
    sl = spec.interior()
    mscale = max(float(np.max(np.abs(Ro[v][sl]))) for v in (1, 2, 3))
    for v in range(5):
        sc = mscale if v in (1, 2, 3) else float(np.max(np.abs(Ro[v][sl])))
        assert float(np.max(np.abs(R[v][sl] - Ro[v][sl]))) < 1e-12 * sc, v


def test_isothermal_wall_refused_outside_its_scope(built_lib):
    """Walls on a face other than y, on a central-scheme block, or without a wall temperature,
    and a stretched y grid without walls on both y faces or without viscous terms, are refused
    at osb_block_add."""
    from opensbli_gb300.solver import Solver
    spec, q = problems.channel_iso((16, 17, 8))
    bad = []
    s1 = problems.channel_iso((16, 17, 8))[0]
    s1.wall_temperature = {(1, 0): 0.0, (1, 1): 1.0}
    bad.append(s1)
    s2 = problems.channel_iso((16, 17, 8))[0]
    s2.scheme = abi.SCHEME_CENTRAL4
    bad.append(s2)
    s3 = problems.channel_iso((16, 17, 8))[0]
    s3.bc = [[abi.BC_ISOTHERMAL_WALL] * 2, [abi.BC_PERIODIC] * 2, [abi.BC_PERIODIC] * 2]
    s3.wall_temperature = {(0, 0): 1.0, (0, 1): 1.0}
    bad.append(s3)
    # a stretched y grid needs walls on both y faces and viscous terms
    s4 = problems.channel_iso((16, 17, 8), stretch=1.7)[0]
    s4.bc = [[abi.BC_PERIODIC] * 2, [abi.BC_PERIODIC] * 2, [abi.BC_PERIODIC] * 2]
    bad.append(s4)
    s5 = problems.channel_iso((16, 17, 8), stretch=1.7)[0]
    s5.viscous = abi.VISC_NONE
    bad.append(s5)
    for sp in bad:
        with pytest.raises(abi.OSBError):
            Solver([(sp, q)], precision="fp64", rk="ls3")
