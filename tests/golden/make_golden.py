"""Generate the golden vectors in tests/golden/ from the reference's own generated solvers.

Needs the reference checkout (to regenerate oracle/_ref) and g++.  For every case the
initial state and the states after 1 stage, 1 step and several steps are written from the
output of the reference solver (OPS C++ generated by OpenSBLI, compiled with
oracle/ops_compat.h), interior points only, FP64, as a compressed .npz:

    python tests/golden/make_golden.py            # all cases
    python tests/golden/make_golden.py tvd        # the TVD-filtered TGV
"""
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import harness  # noqa: E402
from opensbli_gb300 import abi, problems  # noqa: E402


def perturb(q, amp, seed):
    rng = np.random.default_rng(seed)
    return [a * (1.0 + amp * rng.standard_normal(a.shape)) for a in q]


CASES = {
    # name: (reference case, problem builder, env, dt, stage counts, perturbation)
    "sod_extrap_200_perturbed": ("sod_extrap", lambda: problems.sod(200, bc=(abi.BC_EXTRAP1, abi.BC_EXTRAP0)),
                                 {"OSB_NP0": 200}, 2e-4, [1, 3, 30], (1e-2, 13)),
    "sod_weno5js_400": ("sod_weno5js", lambda: problems.sod(400), {"OSB_NP0": 400}, 2e-4, [1, 3, 30, 3000], None),
    "tgv_teno5_12": ("tgv_teno5", lambda: problems.tgv(12, minf=1.25, scheme=abi.SCHEME_TENO5, averaging=abi.AVG_ROE),
                     {"OSB_NP0": 12, "OSB_NP1": 12, "OSB_NP2": 12}, 1e-3, [1, 3, 12], None),
    "tgv_teno6_12": ("tgv_teno6", lambda: problems.tgv(12, minf=1.25, scheme=abi.SCHEME_TENO6, averaging=abi.AVG_ROE),
                     {"OSB_NP0": 12, "OSB_NP1": 12, "OSB_NP2": 12}, 1e-3, [1, 3, 12], None),
    "tgv_weno5z_12_perturbed": ("tgv_weno5z",
                                lambda: problems.tgv(12, minf=1.25, scheme=abi.SCHEME_WENO5_Z),
                                {"OSB_NP0": 12, "OSB_NP1": 12, "OSB_NP2": 12}, 1e-3, [1, 3], (1e-3, 11)),
    "tgv_central_12": ("tgv_central", lambda: problems.tgv(12, minf=0.1, scheme=abi.SCHEME_CENTRAL4),
                       {"OSB_NP0": 12, "OSB_NP1": 12, "OSB_NP2": 12}, 3.385e-3, [1, 3, 30], None),
    "kh_weno5z_24_perturbed": ("kh_weno5z", lambda: problems.kh(24, amp=1.0, phase=0.0),
                               {"OSB_NP0": 24, "OSB_NP1": 24}, 2e-4, [1, 3, 6], (1e-3, 12)),
    "shock_reflection_64x32_perturbed": ("shock_reflection", lambda: problems.shock_reflection(64, 32),
                                         {"OSB_NP0": 64, "OSB_NP1": 32}, 0.5, [1, 3, 30], (1e-2, 4)),
    # the same with the app's own three-stage SSP coefficients
    "shock_reflection_ssp_64x32_perturbed": ("shock_reflection_ssp", lambda: problems.shock_reflection(64, 32),
                                             {"OSB_NP0": 64, "OSB_NP1": 32}, 0.5, [1, 3, 30], (1e-2, 4)),
    # the app's own HLLC-LM flux with its SSP RK3
    "shock_reflection_hllc_64x32_perturbed": ("shock_reflection_hllc",
                                              lambda: problems.shock_reflection(64, 32, flux_type=abi.FLUX_HLLC_LM),
                                              {"OSB_NP0": 64, "OSB_NP1": 32}, 0.5, [1, 3, 30], (1e-2, 4)),
    # PressureOutletBC (back pressure 0.2) in place of the extrapolation outlet
    "shock_reflection_pout_64x32_perturbed": ("shock_reflection_pout",
                                              lambda: problems.shock_reflection(64, 32, back_pressure=0.2),
                                              {"OSB_NP0": 64, "OSB_NP1": 32}, 0.5, [1, 3, 30], (1e-2, 4)),
    # the curvilinear solver computes its metrics from its own grid; they match
    # problems.metrics_central4 bit for bit
    "curv_weno5z_32": ("curv_weno5z", lambda: problems.curvilinear_wave_2d(32),
                       {"OSB_NP0": 32, "OSB_NP1": 32}, 5e-4, [1, 3, 30], None),
    # isothermal no-slip walls on both y faces with the Carpenter closures of the viscous terms
    "channel_iso_16x17x8_perturbed": ("channel_iso", lambda: problems.channel_iso((16, 17, 8)),
                                      {"OSB_NP0": 16, "OSB_NP1": 17, "OSB_NP2": 8}, 1e-3, [1, 3, 30],
                                      (1e-3, 41)),
    # the same with the upper wall adiabatic
    "channel_adi_16x17x8_perturbed": ("channel_adi", lambda: problems.channel_iso((16, 17, 8), upper="adiabatic"),
                                      {"OSB_NP0": 16, "OSB_NP1": 17, "OSB_NP2": 8}, 1e-3, [1, 3, 30],
                                      (1e-3, 42)),
    # the isothermal channel on the stretched wall-normal grid of the TENO turbulent-channel app
    # (MetricsEquation stretched in y, applied to the equations); the solver's own D11 / SD111
    # rows are stored with the states
    "channel_str_16x17x8_perturbed": ("channel_str", lambda: problems.channel_iso((16, 17, 8), stretch=1.7),
                                      {"OSB_NP0": 16, "OSB_NP1": 17, "OSB_NP2": 8}, 1e-3, [1, 3, 30],
                                      (1e-3, 43)),
    # the TENO turbulent-channel app's discretisation (TENO6, power-law viscosity, constant
    # forcing, stretched wall-normal grid, SSP RK3)
    "channel_tcf_16x17x8_perturbed": ("channel_tcf", lambda: problems.channel_tcf((16, 17, 8)),
                                      {"OSB_NP0": 16, "OSB_NP1": 17, "OSB_NP2": 8}, 2e-4, [1, 3, 30],
                                      (1e-3, 44)),
    # the SBLI apps' inflow / outflow faces: the pressure-extrapolation inlet (subsonic and
    # supersonic branch) and the extrapolation outlet, with the viscous terms' closures at both
    "duct_inlet_sub_20x17x8_perturbed": ("duct_inlet_sub", lambda: problems.duct_inlet((20, 17, 8), minf=0.5),
                                         {"OSB_NP0": 20, "OSB_NP1": 17, "OSB_NP2": 8}, 5e-4, [1, 3, 30],
                                         (1e-3, 45)),
    "duct_inlet_sup_20x17x8_perturbed": ("duct_inlet_sup", lambda: problems.duct_inlet((20, 17, 8), minf=2.0),
                                         {"OSB_NP0": 20, "OSB_NP1": 17, "OSB_NP2": 8}, 5e-4, [1, 3, 30],
                                         (1e-3, 46)),
    # the Katzer SBLI app's discretisation: 2D WENO5-Z + viscous terms (Sutherland ratio law),
    # inlet, extrapolation outlet, isothermal wall, Dirichlet top, sinh-stretched y, SSP RK3
    "katzer_24x17_perturbed": ("katzer", lambda: problems.katzer((24, 17)), {"OSB_NP0": 24, "OSB_NP1": 17}, 0.04,
                               [1, 3, 30], (1e-3, 47)),
    # 3D curvilinear TENO5 (MetricsEquation, every direction curvilinear); the solver's own metric
    # arrays are stored with the states (interior; their halos are the periodic images)
    "curv3d_teno5_16x12x10_perturbed": ("curv3d_teno5", lambda: problems.curvilinear_wave_3d((16, 12, 10)),
                                        {"OSB_NP0": 16, "OSB_NP1": 12, "OSB_NP2": 10}, 2e-3, [1, 3, 30],
                                        (1e-3, 21)),
}

METRIC_NAMES = ["D00", "D01", "D02", "D10", "D11", "D12", "D20", "D21", "D22", "detJ"]


def make(name):
    case, mk, env, dt, counts, pert = CASES[name]
    spec, q, *met = mk()
    if pert is not None:
        q = perturb(q, *pert)
    ob = harness.OracleBlocks([(spec, q) + tuple(met)])
    ob.apply_bc()  # periodic images / boundary values exactly as the reference's exchanges
    names = harness.state_names(spec.ndim)
    init = {n: ob.q[0][v] for v, n in enumerate(names)}
    sl = spec.interior()
    out = {"ic": np.stack([ob.q[0][v][sl] for v in range(spec.nvars)]), "dt": dt,
           "counts": np.array(counts)}
    e = dict(env)
    e["OSB_DT"] = repr(dt)
    e["OSB_NITER"] = max(counts) // 3 + 1
    for n in counts:
        r = harness.run_ref(case, env=e, init=init, stop_after_rk=n)
        out["after_%d" % n] = np.stack([r[nm][sl] for nm in names])
        if n == 1 and "Residual0_B0" in r:
            out["residual_1"] = np.stack([r["Residual%d_B0" % v][sl] for v in range(spec.nvars)])
        if n == 1 and spec.ystretch is not None:
            h = spec.halo
            rows = slice(h, h + spec.size[1])
            line = (slice(h, h + 1), rows, slice(h, h + 1)) if spec.ndim == 3 else (rows, slice(h, h + 1))
            out["ystretch"] = np.stack([r[m][line].reshape(-1) for m in ("D11_B0", "SD111_B0")])
            for m in ("D11_B0", "SD111_B0"):  # a function of the row only
                a = r[m][sl]
                first = a[:1, :, :1] if spec.ndim == 3 else a[:, :1]
                assert np.array_equal(a, np.broadcast_to(first, a.shape))
        elif n == 1 and spec.ndim == 3 and "detJ_B0" in r:
            mets = [r[m + "_B0"] for m in METRIC_NAMES]
            for m in mets:  # the generated solver exchanges its metrics periodically
                b = np.zeros_like(m)
                b[sl] = m[sl]
                problems._periodic_fill(spec, b, spec.halo)
                assert np.array_equal(b[2:-2, 2:-2, 2:-2], m[2:-2, 2:-2, 2:-2])
            out["metrics"] = np.stack([m[sl] for m in mets])
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print("wrote", name)


def make_shipped_teno6(n=12, counts=(1, 3, 15)):
    """Golden states from the reference's shipped TENO6 benchmark solver itself (bit-exact
    generated code, apps/performance_benchmark/TENO6), strong-scaling mode at n^3."""
    spec, q = problems.tgv(n, minf=1.25, scheme=abi.SCHEME_TENO6, averaging=abi.AVG_ROE)
    names = harness.state_names(3)
    sl = spec.interior()
    out = {"dt": 0.00084625 * 256 / n, "counts": np.array(counts)}
    for c in counts:
        r = harness.run_shipped_teno6(n, c // 3 + 1, stop_after_rk=c)
        out["after_%d" % c] = np.stack([r[nm][sl] for nm in names])
    np.savez_compressed(os.path.join(HERE, "shipped_teno6_%d.npz" % n), **out)
    print("wrote shipped_teno6_%d" % n)


def c4w5_spec(n):
    """The Central4-WENO5 benchmark's block: supersonic TGV, central-4 KGP convective terms,
    Sutherland viscosity, WENO3 filter with Ducros_check = Ducros_select = 0.05."""
    spec, q = problems.tgv(n, minf=1.25, scheme=abi.SCHEME_CENTRAL4, viscous=abi.VISC_SUTHERLAND)
    spec.split_form = abi.SPLIT_KGP
    spec.filter = abi.FILTER_WENO3
    spec.ducros_check = 0.05
    spec.ducros_select = 0.05
    return spec, q


def make_shipped_c4w5(n=16, steps=(1, 2, 5)):
    """Golden states from the reference's shipped Central4-WENO5 benchmark solver itself
    (bit-exact generated code, apps/performance_benchmark/Central4-WENO5), strong-scaling mode
    at n^3, dumped at exit after whole filtered steps; also the filter mask of the first step."""
    spec, q = c4w5_spec(n)
    names = harness.state_names(3)
    sl = spec.interior()
    out = {"dt": 0.00084625 * 256 / n, "steps": np.array(steps)}
    for c in steps:
        r = harness.run_shipped("c4w5", n, c)
        out["after_%d" % c] = np.stack([r[nm][sl] for nm in names])
        if c == 1:
            out["mask_1"] = r["WENO_filter_B0"][sl]
            out["kappa_1"] = r["kappa_B0"][sl]
    np.savez_compressed(os.path.join(HERE, "shipped_c4w5_%d.npz" % n), **out)
    print("wrote shipped_c4w5_%d" % n)


def make_tvd(n=12, steps=(1, 2, 4), dt=2e-3, kappa=1.25, pert=(2e-2, 5)):
    """Golden states of the generated solver of the TGV app's TVD branch (reference case
    tgv_kgp_tvd: central KGP + Sutherland viscous terms, RK-LS3, TVD filter after every step),
    dumped at exit after whole steps, from a perturbed TGV state."""
    spec, q = problems.tgv_tvd(n, kappa=kappa)
    q = perturb(q, *pert)
    ob = harness.OracleBlocks([(spec, q)])
    ob.apply_bc()
    names = harness.state_names(3)
    init = {nm: ob.q[0][v] for v, nm in enumerate(names)}
    sl = spec.interior()
    out = {"ic": np.stack([ob.q[0][v][sl] for v in range(5)]), "dt": dt, "kappa": kappa,
           "steps": np.array(steps), "pert": np.array(pert)}
    for c in steps:
        env = {"OSB_NP0": n, "OSB_NP1": n, "OSB_NP2": n, "OSB_DT": repr(dt), "OSB_NITER": c,
               "OSB_KAPPA_TVD": repr(kappa)}
        r = harness.run_ref("tgv_kgp_tvd", env=env, init=init)
        out["after_%d" % c] = np.stack([r[nm][sl] for nm in names])
    name = "tgv_kgp_tvd_%d_perturbed" % n
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print("wrote", name)


def make_mb2_flip(sizes=(24, 20), counts=(1, 3, 30), dt=5e-4, pert=(1e-3, 31)):
    """Golden states of the generated two-block case with flipped interfaces (reference case
    mb2_flip: MultiBlock, TraditionalAlgorithmRKMB), from perturbed states of both blocks."""
    blocks = problems.flipped_pair_2d(sizes)
    blocks = [(s, perturb(q, *pert)) for s, q in blocks]
    ob = harness.OracleBlocks(blocks)
    ob.apply_bc()
    init = {}
    for b in range(2):
        for v, nm in enumerate(["rho", "rhou0", "rhou1", "rhoE"]):
            init["%s_B%d" % (nm, b)] = ob.q[b][v]
    out = {"dt": dt, "counts": np.array(counts), "pert": np.array(pert)}
    sl = blocks[0][0].interior()
    for b in range(2):
        out["ic_%d" % b] = np.stack([ob.q[b][v][sl] for v in range(4)])
    env = {"OSB_NP0": sizes[0], "OSB_NP1": sizes[1], "OSB_DT": repr(dt), "OSB_NITER": max(counts) // 3 + 1}
    for n in counts:
        # the harness counts every block's update: a stage of the two blocks is two updates
        r = harness.run_ref("mb2_flip", env=env, init=init, stop_after_rk=2 * n)
        for b in range(2):
            out["after_%d_%d" % (n, b)] = np.stack([r["%s_B%d" % (nm, b)][sl] for nm in ["rho", "rhou0", "rhou1", "rhoE"]])
    name = "mb2_flip_%dx%d_perturbed" % sizes
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print("wrote", name)


def main():
    if sys.argv[1:] == ["mb2_flip"]:
        make_mb2_flip()
        return
    if sys.argv[1:] == ["tvd"]:
        if not harness.ref_available("tgv_kgp_tvd"):
            subprocess.check_call([sys.executable, os.path.join(ROOT, "oracle", "ref_generate.py"), "tgv_kgp_tvd"])
        make_tvd()
        return
    if sys.argv[1:] == ["shipped_teno6"]:
        make_shipped_teno6()
        return
    if sys.argv[1:] == ["shipped_c4w5"]:
        make_shipped_c4w5()
        return
    missing = sorted({c for c in harness_cases() if not harness.ref_available(c)})
    if missing:
        subprocess.check_call([sys.executable, os.path.join(ROOT, "oracle", "ref_generate.py")] + missing)
    for name in (sys.argv[1:] or CASES):
        make(name)


def harness_cases():
    return [c[0] for c in CASES.values()]


if __name__ == "__main__":
    main()
