"""The drop-in seam end to end on the GPU: the reference's own problem definitions, as
GB300Backend maps them (the plans under tests/golden/, which tests/test_backend.py pins to the
reference's scripts), are initialised and run through GB300Backend.from_plan(...).initialise()
.run() -- the path a user script takes after swapping OPSC(alg) for GB300Backend(alg) -- and
compared with the oracle advanced from the same initial state (FP64, 1e-12 relative), with
the reference's own generated solver (golden states) and with its published known answer."""
import os

import numpy as np
import pytest

from opensbli_gb300 import abi

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _plan(name):
    from opensbli_gb300.backend import BackendPlan
    return BackendPlan.load(os.path.join(GOLDEN, "plan_%s.npz" % name))


def _run(name, precision="fp64"):
    from opensbli_gb300.backend import GB300Backend
    plan = _plan(name)
    be = GB300Backend.from_plan(plan, precision=precision).initialise().run()
    got = [be.state(i) for i in range(len(plan.specs))]
    met = [None if m is None else [None if a is None else a.cpu().numpy() for a in m] for m in be.metrics]
    be.close()
    return plan, got, met


def _oracle(plan, met):
    import harness
    items = [(s, q) if m is None else (s, q, m) for s, q, m in zip(plan.specs, plan.states, met)]
    ob = harness.OracleBlocks(items)
    ob.apply_bc()
    ob.step(plan.rk[0], plan.rk[1], plan.rk[2], plan.dt, plan.niter)
    return ob


@pytest.mark.parametrize("name", ["sod400", "tgv_teno5_12", "curv128", "curv3d_16x12x10", "shock_64x32", "kh_32",
                                  "mb2_flip", "channel_iso", "channel_adi", "channel_str", "channel_tcf"])
def test_backend_plan_runs_like_the_oracle(built_lib, oracle_lib, name):
    import harness
    plan, got, met = _run(name)
    ob = _oracle(plan, met)
    for ib, spec in enumerate(plan.specs):
        sl = spec.interior()
        errs = [harness.rel_err(got[ib][v][sl], ob.q[ib][v][sl]) for v in range(spec.nvars)]
        # the unperturbed KH state has flat bands where WENO5-Z's smoothness ratios are rounding
        # noise (epsilon 1e-40), so its parity is stated at 1e-10, as for the KH cases of
        # test_gpu_parity.py
        tol = {"sod400": 1e-11, "kh_32": 1e-10}.get(name, 1e-12)
        assert max(errs) < tol, (name, errs)


def test_backend_curvilinear_known_answer(built_lib):
    """The reference's curvilinear verification case through the backend, metrics generated on
    the GPU from the script's own coordinates: rho at [69, 69] of the halo-inclusive array after
    10 steps on 128^2 is 0.9984292346559068 to 1e-9
    (tests/verification_apps/euler_wave_curvilinear/check_opensbli_output.py)."""
    plan, got, met = _run("curv128")
    assert plan.specs[0].curvilinear and met[0] is not None
    rho = got[0][0][69, 69]
    assert abs(rho - 0.9984292346559068) < 1e-9 * 0.9984292346559068, rho


def test_backend_sod_matches_reference_solver(built_lib):
    """Sod 400 through the backend for the script's 1000 steps against the reference's generated
    solver (golden state after 3000 stages)."""
    import harness
    plan, got, _ = _run("sod400")
    g = np.load(os.path.join(GOLDEN, "sod_weno5js_400.npz"))
    sl = plan.specs[0].interior()
    errs = [harness.rel_err(got[0][v][sl], g["after_3000"][v]) for v in range(3)]
    assert max(errs) < 1e-11, errs


def test_backend_curvilinear_3d_metrics_match_reference(built_lib):
    """The metric arrays the backend generates on the GPU (osb_metrics) for the 3D curvilinear
    script against the reference solver's own (golden, adj(J)/det J in its operation order):
    1e-13 relative."""
    from test_oracle_golden import reference_metrics
    plan, _, met = _run("curv3d_16x12x10")
    spec = plan.specs[0]
    ref = reference_metrics(spec)
    sl = spec.interior()
    for k in range(10):
        scale = float(np.max(np.abs(ref[k][sl])))
        assert float(np.max(np.abs(met[0][k][sl] - ref[k][sl]))) < 1e-13 * scale, k


def test_backend_fp32_residual_plan(built_lib):
    """The same plan in the FP32-residual mode stays within the FP32 tolerance of the FP64 run."""
    import harness
    _, g64, _ = _run("tgv_teno5_12")
    plan, g32, _ = _run("tgv_teno5_12", precision="fp32")
    sl = plan.specs[0].interior()
    errs = [harness.rel_err(g32[0][v][sl], g64[0][v][sl]) for v in (0, 4)]
    assert max(errs) < 1e-5, errs


def test_curvilinear_plan_without_coordinates_is_refused(built_lib):
    from opensbli_gb300.backend import BackendPlan, GB300Backend
    plan = _plan("curv128")
    bad = BackendPlan(plan.specs, plan.states, [None], plan.rk, plan.dt, plan.niter)
    with pytest.raises(abi.OSBError):
        GB300Backend.from_plan(bad).initialise()
