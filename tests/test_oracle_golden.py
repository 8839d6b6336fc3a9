"""The C oracle against the golden vectors produced by the reference's own generated solvers
(tests/golden/make_golden.py).  CPU only."""
import os

import numpy as np
import pytest

import harness
from opensbli_gb300 import abi, problems

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

CURV3D = "curv3d_teno5_16x12x10_perturbed"


def reference_metrics(spec, name=CURV3D):
    """The generated solver's own metric arrays of a golden case (stored on the interior), with
    the periodic halos its exchange gives them."""
    g = np.load(os.path.join(GOLD, name + ".npz"))
    out = []
    for m in g["metrics"]:
        a = np.zeros(spec.shape)
        a[spec.interior()] = m
        problems._periodic_fill(spec, a, spec.halo)
        out.append(a)
    return out


def _curv3d():
    """3D curvilinear TENO5 with the reference solver's own metrics (so the flux path is pinned
    on identical inputs; the metric arrays themselves are compared separately)."""
    spec, q, _, _ = problems.curvilinear_wave_3d((16, 12, 10))
    return spec, q, reference_metrics(spec)


CASES = {
    "sod_weno5js_400": (lambda: problems.sod(400), "ls3", None, 1e-12),
    "sod_extrap_200_perturbed": (lambda: problems.sod(200, bc=(abi.BC_EXTRAP1, abi.BC_EXTRAP0)), "ls3", (1e-2, 13),
                                 1e-12),
    "tgv_teno5_12": (lambda: problems.tgv(12, minf=1.25, scheme=abi.SCHEME_TENO5, averaging=abi.AVG_ROE), "ls3",
                     None, 1e-12),
    "tgv_teno6_12": (lambda: problems.tgv(12, minf=1.25, scheme=abi.SCHEME_TENO6, averaging=abi.AVG_ROE), "ls3",
                     None, 1e-12),
    "tgv_weno5z_12_perturbed": (lambda: problems.tgv(12, minf=1.25, scheme=abi.SCHEME_WENO5_Z), "ls3", (1e-3, 11),
                                1e-11),
    "tgv_central_12": (lambda: problems.tgv(12, minf=0.1, scheme=abi.SCHEME_CENTRAL4), "ls3", None, 1e-12),
    "kh_weno5z_24_perturbed": (lambda: problems.kh(24, amp=1.0, phase=0.0), "sbli3", (1e-3, 12), 1e-9),
    "curv_weno5z_32": (lambda: problems.curvilinear_wave_2d(32), "ls3", None, 1e-12),
    # 3D curvilinear TENO5 (MetricsEquation + LFTeno(5)), the 4-block configuration's discretisation
    CURV3D: (_curv3d, "ls3", (1e-3, 21), 1e-12),
    # Dirichlet inlet and top (post-shock state from x = 40), extrapolation outlet, symmetry wall
    "shock_reflection_64x32_perturbed": (lambda: problems.shock_reflection(64, 32), "ls3", (1e-2, 4), 1e-12),
    "shock_reflection_ssp_64x32_perturbed": (lambda: problems.shock_reflection(64, 32), "ssp3", (1e-2, 4), 1e-12),
    # HLLC-LM flux from WENO5-Z reconstructed states (the app's own flux)
    "shock_reflection_hllc_64x32_perturbed": (lambda: problems.shock_reflection(64, 32, flux_type=abi.FLUX_HLLC_LM),
                                              "ssp3", (1e-2, 4), 1e-12),
    # pressure outlet (back pressure 0.2) in place of the extrapolation outlet
    "shock_reflection_pout_64x32_perturbed": (lambda: problems.shock_reflection(64, 32, back_pressure=0.2), "ls3",
                                              (1e-2, 4), 1e-12),
    # isothermal no-slip walls (both y faces) with the Carpenter closures of the viscous terms
    "channel_iso_16x17x8_perturbed": (lambda: problems.channel_iso((16, 17, 8)), "ls3", (1e-3, 41), 1e-12),
    "channel_adi_16x17x8_perturbed": (lambda: problems.channel_iso((16, 17, 8), upper="adiabatic"), "ls3",
                                      (1e-3, 42), 1e-12),
    # the same on the stretched wall-normal grid of the TENO turbulent-channel app (D11 / SD111)
    "channel_str_16x17x8_perturbed": (lambda: _channel_str(), "ls3", (1e-3, 43), 1e-12),
    # the TENO turbulent-channel app's discretisation: TENO6, power-law viscosity, constant
    # forcing, stretched wall-normal grid, SSP RK3
    "channel_tcf_16x17x8_perturbed": (lambda: _channel_tcf(), "ssp3", (1e-3, 44), 1e-12),
    # the SBLI apps' pressure-extrapolation inlet (subsonic / supersonic branch) and extrapolation
    # outlet on a walled duct, the viscous terms' closures at all four faces
    "duct_inlet_sub_20x17x8_perturbed": (lambda: problems.duct_inlet((20, 17, 8), minf=0.5), "ls3", (1e-3, 45),
                                         1e-12),
    "duct_inlet_sup_20x17x8_perturbed": (lambda: problems.duct_inlet((20, 17, 8), minf=2.0), "ls3", (1e-3, 46),
                                         1e-12),
    # the Katzer SBLI app's discretisation (2D; inlet, extrapolation outlet, isothermal wall and
    # Dirichlet top, all with closures; sinh-stretched y; Sutherland's ratio law; SSP RK3)
    "katzer_24x17_perturbed": (lambda: _katzer(), "ssp3", (1e-3, 47), 1e-12),
}


OUTLET_PLANE_OVERWRITTEN = {"shock_reflection_pout_64x32_perturbed"}


def _channel_str(sizes=(16, 17, 8), stretch=1.7):
    """The stretched channel with the oracle's own wall-normal metrics (oracle_ystretch_metrics
    of the grid line) in place of the library's."""
    spec, q = problems.channel_iso(sizes, stretch=stretch)
    spec.ystretch = harness.ystretch_metrics(problems.stretched_line(sizes[1], stretch), spec.delta[1])
    return spec, q


def _channel_tcf(sizes=(16, 17, 8), stretch=1.7):
    """The TENO channel app's case with the oracle's own wall-normal metrics."""
    spec, q = problems.channel_tcf(sizes, stretch=stretch)
    spec.ystretch = harness.ystretch_metrics(problems.stretched_line(sizes[1], stretch), spec.delta[1])
    return spec, q


def _katzer(sizes=(24, 17)):
    """The Katzer SBLI case with the oracle's own wall-normal metrics."""
    spec, q = problems.katzer(sizes)
    spec.ystretch = harness.ystretch_metrics(problems.katzer_line(sizes[1]), spec.delta[1])
    return spec, q


def test_ystretch_metrics_match_reference(oracle_lib, built_lib):
    """D11 / SD111 of the stretched grid: the oracle's restatement against the reference solver's
    own arrays (1e-12: the grid line's tanh and the summation order differ at rounding level,
    which the two differentiations amplify to ~1e-13), and the library's osb_ystretch_metrics
    against the oracle (identical)."""
    g = np.load(os.path.join(GOLD, "channel_str_16x17x8_perturbed.npz"))
    line = problems.stretched_line(17, 1.7)
    d = 1.0 / 16.0
    ours = harness.ystretch_metrics(line, d)
    for a, b in zip(ours, g["ystretch"]):
        assert harness.rel_err(a, b) < 1e-12
    lib = abi.ystretch_metrics(line, d)
    for a, b in zip(lib, ours):
        assert np.array_equal(a, b)
    with pytest.raises(ValueError):
        harness.ystretch_metrics(line, d, wall_lo=False)  # no rule for the rows next to a free end


def perturb(q, amp, seed):
    rng = np.random.default_rng(seed)
    return [a * (1.0 + amp * rng.standard_normal(a.shape)) for a in q]


def load_case(name):
    mk, rk, pert, tol = CASES[name]
    spec, q, *met = mk()
    if pert is not None:
        q = perturb(q, *pert)
    return (spec, q) + tuple(met), rk, tol, np.load(os.path.join(GOLD, name + ".npz"))


def rk_params(rk):
    if rk == "ls3":
        return abi.RK_LOW_STORAGE, problems.RK3_LS_A, problems.RK3_LS_B
    if rk == "ssp3":
        return abi.RK_LOW_STORAGE, problems.RK3_SSP_A, problems.RK3_SSP_B
    return abi.RK_SBLI3, problems.RK3_SBLI_NEW, problems.RK3_SBLI_OLD


def advance(ob, spec, rk, dt, nstages):
    kind, A, B = rk_params(rk)
    nsteps, rest = divmod(nstages, 3)
    if nsteps:
        ob.step(kind, A, B, dt, nsteps)
    if rest:
        if kind == abi.RK_SBLI3:
            for v in range(spec.nvars):
                ob.rk[0][v][...] = ob.q[0][v]
        for st in range(rest):
            ob.stage(kind, A, B, st, dt)


@pytest.mark.parametrize("name", sorted(CASES))
def test_initial_state_matches_golden(oracle_lib, name):
    blk, rk, tol, g = load_case(name)
    spec = blk[0]
    ob = harness.OracleBlocks([blk])
    ob.apply_bc()
    sl = spec.interior()
    ic = np.stack([ob.q[0][v][sl] for v in range(spec.nvars)])
    assert np.array_equal(ic, g["ic"])


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_residual_matches_reference(oracle_lib, name):
    blk, rk, tol, g = load_case(name)
    spec = blk[0]
    ob = harness.OracleBlocks([blk])
    ob.apply_bc()
    if "residual_1" not in g:
        pytest.skip("the reference solver of this case keeps no residual arrays")
    R = ob.residual(0)
    sl = spec.interior()
    keep = (slice(None),) * spec.ndim
    if name in OUTLET_PLANE_OVERWRITTEN:
        # the pressure outlet overwrites its boundary plane after every update, so that plane's
        # residual is never used; its stencil holds the outlet's replicated state, whose
        # characteristic jumps are rounding-level, where WENO-Z with epsilon 1e-40 turns
        # rounding differences into 1e-6 relative ones (the states match to 1e-12 regardless)
        keep = (slice(None),) * (spec.ndim - 1) + (slice(0, spec.size[0] - 1),)
    for v in range(spec.nvars):
        assert harness.rel_err(R[v][sl][keep], g["residual_1"][v][keep]) < 10 * tol, v


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_states_match_reference(oracle_lib, name):
    blk, rk, tol, g = load_case(name)
    spec = blk[0]
    dt = float(g["dt"])
    sl = spec.interior()
    for n in g["counts"]:
        n = int(n)
        if n > 300 and os.environ.get("OSB_FAST_TESTS"):
            continue
        ob = harness.OracleBlocks([blk])
        ob.apply_bc()
        advance(ob, spec, rk, dt, n)
        ref = g["after_%d" % n]
        errs = [harness.rel_err(ob.q[0][v][sl], ref[v]) for v in range(spec.nvars)]
        assert max(errs) < (tol if n < 300 else 100 * tol), (n, errs)


def test_curvilinear_known_answer(oracle_lib):
    """The reference's own known answer for its curvilinear Euler verification case
    (tests/verification_apps/euler_wave_curvilinear/check_opensbli_output.py): rho at array
    index [69, 69] of the halo-inclusive 138 x 138 output, after 10 steps of dt 5e-4 on 128^2,
    is 0.9984292346559068 to 1e-9 relative."""
    spec, q, met = problems.curvilinear_wave_2d(128)
    ob = harness.OracleBlocks([(spec, q, met)])
    ob.apply_bc()
    ob.step(abi.RK_LOW_STORAGE, problems.RK3_LS_A, problems.RK3_LS_B, 5e-4, 10)
    rho = ob.q[0][0][69, 69]
    assert abs(rho - 0.9984292346559068) < 1e-9 * 0.9984292346559068, rho


def test_oracle_matches_shipped_teno6_benchmark(oracle_lib):
    """The oracle's TENO6 path against the reference's shipped benchmark solver itself
    (apps/performance_benchmark/TENO6, bit-exact generated code, run in its strong-scaling mode
    at 12^3 by tests/golden/make_golden.py shipped_teno6): 1 stage, 1 step, 5 steps."""
    g = np.load(os.path.join(GOLD, "shipped_teno6_12.npz"))
    spec, q = problems.tgv(12, minf=1.25, scheme=abi.SCHEME_TENO6, averaging=abi.AVG_ROE)
    dt = float(g["dt"])
    sl = spec.interior()
    for n in g["counts"]:
        ob = harness.OracleBlocks([(spec, q)])
        ob.apply_bc()
        advance(ob, spec, "ls3", dt, int(n))
        ref = g["after_%d" % int(n)]
        errs = [harness.rel_err(ob.q[0][v][sl], ref[v]) for v in range(spec.nvars)]
        assert max(errs) < 1e-12, (int(n), errs)


def c4w5_spec(n):
    """The Central4-WENO5 benchmark's block (tests/golden/make_golden.py c4w5_spec)."""
    spec, q = problems.tgv(n, minf=1.25, scheme=abi.SCHEME_CENTRAL4, viscous=abi.VISC_SUTHERLAND)
    spec.split_form = abi.SPLIT_KGP
    spec.filter = abi.FILTER_WENO3
    spec.ducros_check = 0.05
    spec.ducros_select = 0.05
    return spec, q


def test_oracle_matches_shipped_c4w5_benchmark(oracle_lib):
    """The oracle's KGP central convective terms and non-linear WENO3 filter against the
    reference's shipped Central4-WENO5 benchmark solver itself (apps/performance_benchmark/
    Central4-WENO5, bit-exact generated code, strong-scaling mode at 16^3, dumped after 1, 2 and
    5 whole filtered steps by tests/golden/make_golden.py shipped_c4w5).  The filter acts on
    11-15 % of the points there.  Tolerance 1e-11 of each field's scale (rhou2 starts at zero)."""
    g = np.load(os.path.join(GOLD, "shipped_c4w5_16.npz"))
    spec, q = c4w5_spec(16)
    dt = float(g["dt"])
    sl = spec.interior()
    assert 0.05 < float(g["mask_1"].mean()) < 0.5
    for n in g["steps"]:
        ob = harness.OracleBlocks([(spec, q)])
        ob.apply_bc()
        ob.step(abi.RK_LOW_STORAGE, problems.RK3_LS_A, problems.RK3_LS_B, dt, int(n))
        ref = g["after_%d" % int(n)]
        errs = [harness.rel_err(ob.q[0][v][sl], ref[v]) for v in range(spec.nvars)]
        assert max(errs) < 1e-11, (int(n), errs)


def test_kgp_differs_from_feiereisen(oracle_lib):
    """The split form is honoured: the same state gives different convective residuals."""
    spec, q = c4w5_spec(12)
    ob = harness.OracleBlocks([(spec, q)])
    ob.apply_bc()
    r_kgp = ob.residual(0)
    spec.split_form = abi.SPLIT_FEIEREISEN
    ob2 = harness.OracleBlocks([(spec, q)])
    ob2.apply_bc()
    r_f = ob2.residual(0)
    sl = spec.interior()
    assert harness.rel_err(r_kgp[0][sl], r_f[0][sl]) > 1e-3


def tvd_case():
    """The TVD-filtered TGV of tests/golden/make_golden.py make_tvd: the perturbed initial
    state and the golden states of the reference's generated solver."""
    g = np.load(os.path.join(GOLD, "tgv_kgp_tvd_12_perturbed.npz"))
    spec, q = problems.tgv_tvd(12, kappa=float(g["kappa"]))
    amp, seed = g["pert"]
    return spec, perturb(q, float(amp), int(seed)), g


def test_oracle_matches_reference_tvd_filter(oracle_lib):
    """The oracle's non-linear TVD filter (with the KGP central step before it) against the
    reference's own generated solver of the TGV app's TVD branch (oracle/ref_generate.py case
    tgv_kgp_tvd, compiled with oracle/ops_compat.h), after 1, 2 and 4 whole filtered steps from a
    perturbed state: 1e-13 of each field's scale.  The filter moves the state by about 2e-3 of
    its scale per step here, so the comparison sees it (an unfiltered step misses by 1e-3)."""
    spec, q, g = tvd_case()
    dt = float(g["dt"])
    sl = spec.interior()
    ob = harness.OracleBlocks([(spec, q)])
    ob.apply_bc()
    assert np.array_equal(np.stack([ob.q[0][v][sl] for v in range(5)]), g["ic"])
    for n in g["steps"]:
        ob = harness.OracleBlocks([(spec, q)])
        ob.apply_bc()
        ob.step(abi.RK_LOW_STORAGE, problems.RK3_LS_A, problems.RK3_LS_B, dt, int(n))
        ref = g["after_%d" % int(n)]
        errs = [harness.rel_err(ob.q[0][v][sl], ref[v]) for v in range(spec.nvars)]
        assert max(errs) < 1e-13, (int(n), errs)
    # the filter is active: the same step without it is far from the reference
    spec.filter = abi.FILTER_NONE
    ob = harness.OracleBlocks([(spec, q)])
    ob.apply_bc()
    ob.step(abi.RK_LOW_STORAGE, problems.RK3_LS_A, problems.RK3_LS_B, dt, 1)
    assert max(harness.rel_err(ob.q[0][v][sl], g["after_1"][v]) for v in range(5)) > 1e-4


def test_tvd_filter_stale_point_matters(oracle_lib):
    """The generated filter reads u at index -2 left by the last RK stage and a = 0 there; a
    filter that recomputes them from the current state differs from the reference on the planes
    next to the low boundaries (the oracle's standalone filter call takes the current state)."""
    spec, q, g = tvd_case()
    dt = float(g["dt"])
    sl = spec.interior()
    ob = harness.OracleBlocks([(spec, q)])
    ob.apply_bc()
    ob.step(abi.RK_LOW_STORAGE, problems.RK3_LS_A, problems.RK3_LS_B, dt, 1)
    spec.filter = abi.FILTER_NONE
    o2 = harness.OracleBlocks([(spec, q)])
    o2.apply_bc()
    o2.step(abi.RK_LOW_STORAGE, problems.RK3_LS_A, problems.RK3_LS_B, dt, 1)
    o2.desc[0].filter = abi.FILTER_TVD
    o2.filter(dt)
    d = np.abs(ob.q[0][0][sl] - o2.q[0][0][sl])
    assert d[:, :, 0].max() > 1e-8          # x = 0 plane: different
    assert d[2:, 2:, 2:].max() < 1e-13      # away from the low planes: the same


def test_host_metrics_match_reference_3d():
    """The 3D metric arrays from 4th-order central differences of the coordinates
    (problems.metrics_central4: J, then its inverse) against the reference solver's own
    (adj(J) / det J in its generated operation order): equal to rounding, 1e-13 relative."""
    spec, _, met, _ = problems.curvilinear_wave_3d((16, 12, 10))
    ref = reference_metrics(spec)
    sl = spec.interior()
    for k in range(10):
        scale = float(np.max(np.abs(ref[k][sl])))
        assert float(np.max(np.abs(met[k][sl] - ref[k][sl]))) < 1e-13 * scale, k


MB2 = "mb2_flip_24x20_perturbed"


def _mb2_blocks():
    g = np.load(os.path.join(GOLD, MB2 + ".npz"))
    blocks = problems.flipped_pair_2d((24, 20))
    amp, seed = float(g["pert"][0]), int(g["pert"][1])
    blocks = [(s, perturb(q, amp, seed)) for s, q in blocks]
    return blocks, g


def test_flipped_interfaces_match_reference():
    """Two blocks joined by flipped interfaces (InterfaceBC match flag: the neighbour's layers in
    reverse order along the normal), periodic in y: the oracle against the reference's generated
    multi-block solver (MultiBlock + TraditionalAlgorithmRKMB, bc_exchanges with a negative
    to_dir) after 1, 3 and 30 stages, both blocks, 1e-12."""
    blocks, g = _mb2_blocks()
    blocks = [(s, [a for a in q]) for s, q in blocks]
    for n in g["counts"]:
        n = int(n)
        ob = harness.OracleBlocks(blocks)
        ob.apply_bc()
        sl = blocks[0][0].interior()
        if n == 1:
            for b in range(2):
                assert np.array_equal(np.stack([ob.q[b][v][sl] for v in range(4)]), g["ic_%d" % b])
        advance_mb(ob, "ls3", float(g["dt"]), n)
        for b in range(2):
            ref = g["after_%d_%d" % (n, b)]
            errs = [harness.rel_err(ob.q[b][v][sl], ref[v]) for v in range(4)]
            assert max(errs) < 1e-12, (n, b, errs)


def test_flip_matters():
    """Without the flip the same two blocks end elsewhere (the golden states are sensitive to it)."""
    blocks, g = _mb2_blocks()
    for s, _ in blocks:
        s.iface = [[(f[0], f[1], f[2], 0) for f in s.iface[0]], [None, None]]
    ob = harness.OracleBlocks(blocks)
    ob.apply_bc()
    advance_mb(ob, "ls3", float(g["dt"]), 3)
    sl = blocks[0][0].interior()
    assert harness.rel_err(ob.q[0][0][sl], g["after_3_0"][0]) > 1e-6


def advance_mb(ob, rk, dt, nstages):
    kind, A, B = rk_params(rk)
    nsteps, rest = divmod(nstages, 3)
    if nsteps:
        ob.step(kind, A, B, dt, nsteps)
    for st in range(rest):
        ob.stage(kind, A, B, st, dt)
