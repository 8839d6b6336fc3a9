"""The drop-in backend maps OpenSBLI's own problem objects onto block descriptors.  Uses the
upstream generator when its checkout is importable (OSB_REFERENCE), otherwise skips."""
import os

import numpy as np
import pytest

from opensbli_gb300 import abi, problems

import harness  # oracle/ (on the path through conftest): where the upstream checkout lies

REF = harness.reference_root()
needs_ref = pytest.mark.skipif(REF is None, reason="upstream OpenSBLI checkout not available")


def _backend_for(case, numbers):
    import ref_generate
    block, _ = ref_generate.build_case(case, REF)
    from opensbli import TraditionalAlgorithmRK
    from opensbli_gb300.backend import GB300Backend
    import contextlib
    with open(os.devnull, "w") as dn, contextlib.redirect_stdout(dn):
        alg = TraditionalAlgorithmRK(block)
    return GB300Backend(alg, numbers)


TGV_NUMBERS = {"Re": "1600.0", "gama": "1.4", "Pr": "0.71", "dt": "0.001", "niter": "3",
               "block0np0": "16", "block0np1": "16", "block0np2": "16", "Delta0block0": "2*M_PI/block0np0",
               "Delta1block0": "2*M_PI/block0np1", "Delta2block0": "2*M_PI/block0np2", "TENO_CT": "1e-6"}


@needs_ref
@pytest.mark.parametrize("case,scheme,avg,minf", [("tgv_teno5", abi.SCHEME_TENO5, abi.AVG_ROE, 1.25),
                                                  ("tgv_weno5z", abi.SCHEME_WENO5_Z, abi.AVG_SIMPLE, 1.25),
                                                  ("tgv_central", abi.SCHEME_CENTRAL4, abi.AVG_SIMPLE, 0.1)])
def test_tgv_spec_and_initial_state(case, scheme, avg, minf):
    nums = dict(TGV_NUMBERS, Minf=str(minf))
    be = _backend_for(case, nums)
    spec = be.specs[0]
    ref_spec, ref_q = problems.tgv(16, minf=minf, scheme=scheme, averaging=avg)
    assert spec.scheme == ref_spec.scheme and spec.averaging == ref_spec.averaging
    assert spec.viscous == ref_spec.viscous
    assert spec.size == ref_spec.size and np.allclose(spec.delta, ref_spec.delta, rtol=0, atol=0)
    assert spec.bc == ref_spec.bc and spec.bc_depth == ref_spec.bc_depth
    assert be.rk[0] == abi.RK_LOW_STORAGE
    assert np.allclose(be.rk[1], problems.RK3_LS_A) and np.allclose(be.rk[2], problems.RK3_LS_B)
    from opensbli_gb300.backend import initial_state
    q = initial_state(be.blocks[0], spec, nums)
    for v in range(5):
        assert np.allclose(q[v], ref_q[v], rtol=1e-13, atol=1e-13), v


@needs_ref
def test_sod_spec():
    be = _backend_for("sod_weno5js", {"gama": "1.4", "dt": "0.0002", "niter": "1000", "block0np0": "400",
                                      "Delta0block0": "1.0/(block0np0-1)"})
    spec = be.specs[0]
    ref_spec, ref_q = problems.sod(400)
    assert spec.scheme == abi.SCHEME_WENO5_JS and spec.averaging == abi.AVG_SIMPLE
    assert spec.bc == [[abi.BC_ZERO_GRAD, abi.BC_ZERO_GRAD]] and spec.bc_depth == [[4, 4]]
    assert spec.delta[0] == ref_spec.delta[0]
    from opensbli_gb300.backend import initial_state
    q = initial_state(be.blocks[0], spec, {"gama": "1.4", "block0np0": "400", "Delta0block0": "1.0/(block0np0-1)"})
    for v in range(3):
        assert np.array_equal(q[v], ref_q[v]), v


@needs_ref
def test_kh_spec():
    nums = {"gama": "1.4", "dt": "0.0002", "niter": "2", "block0np0": "32", "block0np1": "32",
            "Delta0block0": "1.0/block0np0", "Delta1block0": "1.0/block0np1", "khamp": "1.0", "khphase": "0.0"}
    be = _backend_for("kh_weno5z", nums)
    spec = be.specs[0]
    assert spec.scheme == abi.SCHEME_WENO5_Z and spec.averaging == abi.AVG_ROE
    assert be.rk[0] == abi.RK_SBLI3
    assert spec.bc_depth == [[4, 4], [4, 4]]


@needs_ref
def test_extrapolation_and_teno6_specs():
    be = _backend_for("sod_extrap", {"gama": "1.4", "dt": "0.0002", "niter": "10", "block0np0": "200",
                                     "Delta0block0": "1.0/(block0np0-1)"})
    spec = be.specs[0]
    assert spec.bc == [[abi.BC_EXTRAP1, abi.BC_EXTRAP0]] and spec.bc_depth == [[4, 4]]
    be = _backend_for("tgv_teno6", dict(TGV_NUMBERS, Minf="1.25"))
    assert be.specs[0].scheme == abi.SCHEME_TENO6 and be.specs[0].averaging == abi.AVG_ROE


@needs_ref
def test_precision_follows_reference_datatype_knobs():
    """SimulationDataType (core/datatypes.py:3-17) and OPSC's mixed_precision_config
    (opsc.py:462-534) select the precision mode when none is given."""
    import sys
    import ref_generate
    if REF not in sys.path:
        sys.path.insert(0, REF)
    ref_generate.apply_compat_patches()
    from opensbli.core.datatypes import Double, FloatC, Half, SimulationDataType
    from opensbli_gb300.backend import precision_of
    saved = SimulationDataType.__dict__["dtype"]
    try:
        SimulationDataType.set_datatype(Double)
        assert precision_of() == "fp64"
        assert precision_of({"residuals": ([], FloatC)}) == "fp32"
        assert precision_of({"wk_arrays": ([], FloatC), "RK_arrays": ([], Double)}) == "fp32"
        assert precision_of({"q_vector": ([], Double)}) == "fp64"
        with pytest.raises(NotImplementedError):
            precision_of({"custom": ([], Half)})
        with pytest.raises(ValueError):
            precision_of({"bogus": ([], FloatC)})
        SimulationDataType.set_datatype(FloatC)
        assert precision_of() == "fp32"
        SimulationDataType.set_datatype(Double)
        be = _backend_for("sod_weno5js", {"gama": "1.4", "dt": "0.0002", "niter": "10", "block0np0": "400",
                                          "Delta0block0": "1.0/(block0np0-1)"})
        assert be.precision == "fp64"
    finally:
        setattr(SimulationDataType, "dtype", saved)


TGV_SUPERSONIC = dict(TGV_NUMBERS, Minf="1.25")


@needs_ref
def test_central_split_form_detected():
    """The central scheme's convective split form is read from the block's equations:
    Feiereisen (low-Mach TGV app) and KGP with the enthalpy energy formulation (the central
    branch of compressible_TGV.py) map onto OSB_SPLIT_*; another form fails loudly."""
    be = _backend_for("tgv_central", dict(TGV_NUMBERS, Minf="0.1"))
    assert be.specs[0].split_form == abi.SPLIT_FEIEREISEN
    be = _backend_for("tgv_kgp", TGV_SUPERSONIC)
    spec = be.specs[0]
    assert spec.split_form == abi.SPLIT_KGP and spec.scheme == abi.SCHEME_CENTRAL4
    assert spec.viscous == abi.VISC_SUTHERLAND
    import contextlib
    import ref_generate
    from opensbli import TraditionalAlgorithmRK
    from opensbli_gb300.backend import GB300Backend
    with open(os.devnull, "w") as dn, contextlib.redirect_stdout(dn):
        block, _ = ref_generate.central_split_block("Divergence")
        alg = TraditionalAlgorithmRK(block)
    with pytest.raises(NotImplementedError):
        GB300Backend(alg, TGV_SUPERSONIC)


@needs_ref
def test_tvd_filter_detected():
    """The TVD filter's equation classes (filters/TVD_filter.py, the TGV app's TVD branch) map
    onto OSB_FILTER_TVD with the run's kappa_TVD and the stage exchange depth of its periodic
    BCs; without kappa_TVD the backend refuses the block instead of dropping the filter."""
    be = _backend_for("tgv_kgp_tvd", dict(TGV_SUPERSONIC, kappa_TVD="1.25"))
    spec = be.specs[0]
    ref_spec, _ = problems.tgv_tvd(16, kappa=1.25)
    assert spec.filter == abi.FILTER_TVD and spec.tvd_kappa == 1.25
    assert spec.split_form == abi.SPLIT_KGP and spec.scheme == abi.SCHEME_CENTRAL4
    assert spec.bc_depth == ref_spec.bc_depth
    with pytest.raises(ValueError):
        _backend_for("tgv_kgp_tvd", TGV_SUPERSONIC)
    be = _backend_for("tgv_kgp", TGV_SUPERSONIC)
    assert be.specs[0].filter == abi.FILTER_NONE


@needs_ref
def test_shock_reflection_boundaries_mapped():
    """The shock-reflection app's DirichletBC / ExtrapolationBC / SymmetryBC map onto
    OSB_BC_DIRICHLET (depth = the WENO halo on that side: 3 below, 4 above, as the generated
    ranges), OSB_BC_EXTRAP0 and OSB_BC_SYMMETRY; the Dirichlet faces' values, evaluated from the
    BCs' own equations (the top one from the grid coordinate x0), match problems.shock_reflection
    to rounding (the generated kernel multiplies by 1/(gama-1) where SymPy divides)."""
    nums = {"gama": "1.4", "Minf": "2.0", "dt": "0.1", "niter": "1", "block0np0": "64", "block0np1": "32",
            "Delta0block0": "350.0/(block0np0-1)", "Delta1block0": "115.0/(block0np1-1)"}
    be = _backend_for("shock_reflection", nums)
    spec = be.specs[0]
    ref, q = problems.shock_reflection(64, 32)
    assert spec.bc == ref.bc and spec.bc_depth == ref.bc_depth
    assert spec.scheme == abi.SCHEME_WENO5_Z and spec.averaging == abi.AVG_SIMPLE
    assert sorted(spec.dirichlet) == sorted(ref.dirichlet)
    for k in ref.dirichlet:
        assert spec.dirichlet[k].shape == ref.dirichlet[k].shape, k
        assert np.allclose(spec.dirichlet[k], ref.dirichlet[k], rtol=1e-14, atol=0), k
    from opensbli_gb300.backend import initial_state
    q0 = initial_state(be.blocks[0], spec, nums)
    for v in range(4):
        assert np.allclose(q0[v], q[v], rtol=1e-14, atol=0), v


@needs_ref
def test_hllc_block_maps_and_runs_in_the_oracle():
    """The shock-reflection app with its HLLCWeno (HLLC-LM) flux and SSP RK3 maps onto a
    descriptor with OSB_FLUX_HLLC_LM and the SSP coefficients; the oracle run from the backend's
    own spec and initial state reproduces the reference's generated solver (golden, 30 stages)
    from the same perturbed state."""
    import harness
    nums = {"gama": "1.4", "Minf": "2.0", "dt": "0.5", "niter": "1", "block0np0": "64", "block0np1": "32",
            "Delta0block0": "350.0/(block0np0-1)", "Delta1block0": "115.0/(block0np1-1)"}
    be = _backend_for("shock_reflection_hllc", nums)
    spec = be.specs[0]
    assert spec.flux_type == abi.FLUX_HLLC_LM and spec.scheme == abi.SCHEME_WENO5_Z
    assert be.rk[0] == abi.RK_LOW_STORAGE and np.allclose(be.rk[1], problems.RK3_SSP_A)
    assert np.allclose(be.rk[2], problems.RK3_SSP_B)
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "shock_reflection_hllc_64x32_perturbed.npz"))
    ref_spec, q = problems.shock_reflection(64, 32, flux_type=abi.FLUX_HLLC_LM)
    rng = np.random.default_rng(4)
    q = [a * (1.0 + 1e-2 * rng.standard_normal(a.shape)) for a in q]
    ob = harness.OracleBlocks([(spec, q)])
    ob.apply_bc()
    ob.step(be.rk[0], be.rk[1], be.rk[2], float(g["dt"]), 10)
    sl = spec.interior()
    errs = [harness.rel_err(ob.q[0][v][sl], g["after_30"][v]) for v in range(4)]
    assert max(errs) < 1e-12, errs


@needs_ref
def test_pressure_outlet_maps_and_runs_in_the_oracle():
    """PressureOutletBC maps onto OSB_BC_PRESSURE_OUTLET with its back pressure and depth; the
    oracle run from the backend's own spec reproduces the reference's generated solver."""
    import harness
    nums = {"gama": "1.4", "Minf": "2.0", "dt": "0.5", "niter": "1", "block0np0": "64", "block0np1": "32",
            "Delta0block0": "350.0/(block0np0-1)", "Delta1block0": "115.0/(block0np1-1)"}
    be = _backend_for("shock_reflection_pout", nums)
    spec = be.specs[0]
    ref, q = problems.shock_reflection(64, 32, back_pressure=0.2)
    assert spec.bc == ref.bc and spec.bc_depth == ref.bc_depth and spec.back_pressure == {(0, 1): 0.2}
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "shock_reflection_pout_64x32_perturbed.npz"))
    rng = np.random.default_rng(4)
    q = [a * (1.0 + 1e-2 * rng.standard_normal(a.shape)) for a in q]
    ob = harness.OracleBlocks([(spec, q)])
    ob.apply_bc()
    ob.step(be.rk[0], be.rk[1], be.rk[2], float(g["dt"]), 10)
    sl = spec.interior()
    errs = [harness.rel_err(ob.q[0][v][sl], g["after_30"][v]) for v in range(4)]
    assert max(errs) < 1e-12, errs


PLANS = ["sod400", "tgv_teno5_12", "curv128", "curv3d_16x12x10", "shock_64x32", "kh_32", "mb2_flip", "channel_iso",
         "channel_adi", "channel_str", "channel_tcf"]


@needs_ref
@pytest.mark.parametrize("name", PLANS)
def test_backend_plan_matches_committed_fixture(name):
    """GB300Backend still derives, from the reference's own problem definition, exactly the plan
    committed under tests/golden/ (specs, initial state, coordinates, RK, dt, niter), which the
    GPU tests run through GB300Backend.from_plan.  One interpreter per case: the generator keeps
    module-level state between problems."""
    import subprocess
    import sys
    script = os.path.join(os.path.dirname(__file__), "golden", "make_backend_plans.py")
    r = subprocess.run([sys.executable, script, "--check", name], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]


def test_stretched_channel_plan_is_the_stretched_channel(built_lib):
    """The TENO channel app's stretched wall-normal grid (MetricsEquation stretched in y, applied
    to the equations) as the backend maps it (the committed plan, which
    test_backend_plan_matches_committed_fixture pins to the script): a Cartesian block with the
    D11 / SD111 rows of its grid line, identical to problems.channel_iso(stretch=1.7), and the
    same initial state to rounding."""
    from opensbli_gb300.backend import BackendPlan
    plan = BackendPlan.load(os.path.join(os.path.dirname(__file__), "golden", "plan_channel_str.npz"))
    sp = plan.specs[0]
    spec, q = problems.channel_iso((16, 17, 8), stretch=1.7)
    assert not sp.curvilinear and plan.coords == [None]
    for a, b in zip(sp.ystretch, spec.ystretch):
        assert np.array_equal(a, b)
    for k in ("size", "scheme", "averaging", "viscous", "bc", "bc_depth", "delta", "wall_temperature", "Re", "Minf"):
        assert getattr(sp, k) == getattr(spec, k), k
    sl = spec.interior()
    for v in range(spec.nvars):
        assert np.max(np.abs(plan.states[0][v][sl] - q[v][sl])) <= 1e-15 * np.max(np.abs(q[v][sl])), v


def test_teno_channel_app_plan_is_the_teno_channel(built_lib):
    """The TENO turbulent-channel app's equations as the backend maps them (the committed plan):
    TENO6, the power law mu = T^0.7, the forcing c = (-1, 0, 0) read from its -KD(_i,_j) c_j and
    -Dot(c_j, u_j) terms, the stretched wall-normal grid, the SSP RK3, and the TENO epsilon of the
    generated code (1e-40, not the script's eps parameter): identical to problems.channel_tcf."""
    from opensbli_gb300.backend import BackendPlan
    plan = BackendPlan.load(os.path.join(os.path.dirname(__file__), "golden", "plan_channel_tcf.npz"))
    sp = plan.specs[0]
    spec, q = problems.channel_tcf((16, 17, 8))
    for k in ("size", "scheme", "averaging", "viscous", "visc_power", "forcing", "bc", "delta", "wall_temperature",
              "Re", "Minf", "Pr", "eps", "teno_ct"):
        assert getattr(sp, k) == getattr(spec, k), k
    assert plan.rk[1] == tuple(problems.RK3_SSP_A) and plan.rk[2] == tuple(problems.RK3_SSP_B)
    for a, b in zip(sp.ystretch, spec.ystretch):
        assert np.array_equal(a, b)
    sl = spec.interior()
    for v in range(spec.nvars):
        assert np.max(np.abs(plan.states[0][v][sl] - q[v][sl])) <= 1e-15 * np.max(np.abs(q[v][sl])), v


@needs_ref
def test_curvilinear_script_is_curvilinear():
    """The reference's curvilinear case (MetricsEquation + LFWeno) maps onto a curvilinear spec
    whose coordinates come from its initialisation; the Solver refuses such a spec without
    metric arrays instead of running it as a Cartesian block."""
    be = _backend_for("curv_weno5z", {"gama": "1.4", "dt": "0.0005", "niter": "10", "block0np0": "32",
                                      "block0np1": "32", "Delta0block0": "2.0/(block0np0)",
                                      "Delta1block0": "2.0/(block0np1)"})
    spec = be.specs[0]
    assert spec.curvilinear and be.coord_names[0] == ["x0", "x1"]
    plan = be.plan()
    ref_spec, ref_q, _ = problems.curvilinear_wave_2d(32)
    x0, x1 = problems.wave_2d_coords(ref_spec)
    assert np.array_equal(plan.coords[0][0], x0) and np.array_equal(plan.coords[0][1], x1)
    for v in range(4):
        assert np.array_equal(plan.states[0][v], ref_q[v]), v


@needs_ref
def test_curvilinear_with_non_periodic_faces_refused():
    """A curvilinear block with a non-periodic face needs the one-sided metric closures, which are
    not implemented: the backend refuses it."""
    import contextlib
    import ref_generate
    block, _ = ref_generate.build_case("curv_weno5z", REF)
    from opensbli import TraditionalAlgorithmRK
    from opensbli.core.boundary_conditions.zero_gradient_outlet import ZeroGradientOutletBC
    from opensbli_gb300.backend import GB300Backend
    bts = [list(pair) for pair in block.boundary_types]
    bts[0][1] = ZeroGradientOutletBC(0, 1)
    block.boundary_types = bts
    with open(os.devnull, "w") as dn, contextlib.redirect_stdout(dn):
        alg = TraditionalAlgorithmRK(block)
    with pytest.raises(NotImplementedError, match="Carpenter"):
        GB300Backend(alg, {"gama": "1.4", "block0np0": "32", "block0np1": "32", "Delta0block0": "2.0/(block0np0)",
                           "Delta1block0": "2.0/(block0np1)"})


def test_plan_file_round_trip(tmp_path):
    """BackendPlan.save / load keep every spec field, the Dirichlet faces and the arrays."""
    from opensbli_gb300.backend import BackendPlan
    spec, q = problems.shock_reflection(64, 32)
    cspec, cq, _, x = problems.curvilinear_wave_3d((8, 8, 8))
    plan = BackendPlan([spec, cspec], [q, cq], [None, x], (abi.RK_LOW_STORAGE, problems.RK3_SSP_A,
                                                           problems.RK3_SSP_B), 0.5, 7, "fp32")
    plan.save(str(tmp_path / "p.npz"))
    back = BackendPlan.load(str(tmp_path / "p.npz"))
    assert back.rk == plan.rk and (back.dt, back.niter, back.precision) == (0.5, 7, "fp32")
    for a, b in zip(plan.specs, back.specs):
        ra, xa = a.to_record()
        rb, xb = b.to_record()
        assert ra == rb and sorted(xa) == sorted(xb)
        assert all(np.array_equal(xa[k], xb[k]) for k in xa)
    assert back.specs[1].curvilinear and back.coords[0] is None
    assert all(np.array_equal(u, v) for u, v in zip(back.coords[1], x))
    assert all(np.array_equal(u, v) for u, v in zip(back.states[0], q))
