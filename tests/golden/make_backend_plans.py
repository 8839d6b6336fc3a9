"""Generate the backend plans in tests/golden/plan_*.npz from the reference's own problem
definitions.

Each case builds an OpenSBLI problem with the reference's Python API (oracle/ref_generate.py),
hands its algorithm to GB300Backend as a user script would in place of OPSC(alg), and saves
the BackendPlan the backend derives from it: block specs (schemes, boundaries, constants,
curvilinear flag), the initial state the script's GridBasedInitialisation evaluates to, the
grid coordinates of curvilinear blocks, the time integrator, dt and niter.  The GPU tests run
these plans through GB300Backend.from_plan where the OpenSBLI generator is not installed;
tests/test_backend.py checks, where the reference checkout is present, that the backend still
derives exactly these plans.

    python tests/golden/make_backend_plans.py            # all cases
    python tests/golden/make_backend_plans.py curv128    # one case
    python tests/golden/make_backend_plans.py --check curv128   # exit 1 if the plan changed
"""
import contextlib
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

TGV = {"Re": "1600.0", "gama": "1.4", "Pr": "0.71", "Minf": "1.25", "dt": "0.001", "niter": "4",
       "block0np0": "12", "block0np1": "12", "block0np2": "12", "Delta0block0": "2*M_PI/block0np0",
       "Delta1block0": "2*M_PI/block0np1", "Delta2block0": "2*M_PI/block0np2", "TENO_CT": "1e-6"}

# plan name: (reference case of oracle/ref_generate.py, simulation parameters of the run)
CASES = {
    # Sod tube, WENO5-JS, zero-gradient ends, 1000 steps (the 1D benchmark configuration)
    "sod400": ("sod_weno5js", {"gama": "1.4", "dt": "0.0002", "niter": "1000", "block0np0": "400",
                               "Delta0block0": "1.0/(block0np0-1)"}),
    # supersonic TGV, TENO5 (Roe average) + central viscous terms, 12^3
    "tgv_teno5_12": ("tgv_teno5", TGV),
    # wavy-mesh curvilinear Euler wave, WENO5-Z: the verification case and its known answer
    # rho_B0[69,69] after 10 steps of dt 5e-4 on 128^2
    "curv128": ("curv_weno5z", {"gama": "1.4", "dt": "0.0005", "niter": "10", "block0np0": "128",
                                "block0np1": "128", "Delta0block0": "2.0/(block0np0)",
                                "Delta1block0": "2.0/(block0np1)"}),
    # 3D wavy-mesh curvilinear Euler, TENO5 (Roe average), metrics from the script's MetricsEquation
    "curv3d_16x12x10": ("curv3d_teno5", {"gama": "1.4", "Minf": "0.7", "dt": "0.002", "niter": "5",
                                         "TENO_CT": "1e-6", "block0np0": "16", "block0np1": "12", "block0np2": "10",
                                         "Delta0block0": "1.0/(block0np0)", "Delta1block0": "1.0/(block0np1)",
                                         "Delta2block0": "1.0/(block0np2)"}),
    # inviscid shock reflection: Dirichlet, symmetry and extrapolation faces
    "shock_64x32": ("shock_reflection", {"gama": "1.4", "Minf": "2.0", "dt": "0.5", "niter": "10",
                                         "block0np0": "64", "block0np1": "32",
                                         "Delta0block0": "350.0/(block0np0-1)", "Delta1block0": "115.0/(block0np1-1)"}),
    # two blocks joined by flipped interfaces (MultiBlock, TraditionalAlgorithmRKMB)
    "mb2_flip": ("mb2_flip", {"gama": "1.4", "dt": "0.0005", "niter": "10",
                              "block0np0": "24", "block0np1": "20", "Delta0block0": "1.0/block0np0",
                              "Delta1block0": "1.0/block0np1", "block1np0": "24", "block1np1": "20",
                              "Delta0block1": "1.0/block1np0", "Delta1block1": "1.0/block1np1"}),
    # 3D channel between isothermal no-slip walls (TENO5 + viscous terms with the Carpenter closures)
    "channel_iso": ("channel_iso", {"Re": "100.0", "gama": "1.4", "Minf": "0.5", "Pr": "0.71", "Twall": "1.0",
                                    "dt": "0.001", "niter": "10", "TENO_CT": "1e-6", "block0np0": "16",
                                    "block0np1": "17", "block0np2": "8", "Delta0block0": "2*M_PI/block0np0",
                                    "Delta1block0": "2.0/(block0np1-1)", "Delta2block0": "2*M_PI/block0np2"}),
    # the same channel with the upper wall adiabatic
    "channel_adi": ("channel_adi", {"Re": "100.0", "gama": "1.4", "Minf": "0.5", "Pr": "0.71", "Twall": "1.0",
                                    "dt": "0.001", "niter": "10", "TENO_CT": "1e-6", "block0np0": "16",
                                    "block0np1": "17", "block0np2": "8", "Delta0block0": "2*M_PI/block0np0",
                                    "Delta1block0": "2.0/(block0np1-1)", "Delta2block0": "2*M_PI/block0np2"}),
    # the isothermal channel on the stretched wall-normal grid of the TENO turbulent-channel app
    # (MetricsEquation stretched in y, applied to the equations)
    "channel_str": ("channel_str", {"Re": "100.0", "gama": "1.4", "Minf": "0.5", "Pr": "0.71", "Twall": "1.0",
                                    "stretch": "1.7", "dt": "0.001", "niter": "10", "TENO_CT": "1e-6",
                                    "block0np0": "16", "block0np1": "17", "block0np2": "8",
                                    "Delta0block0": "2*M_PI/block0np0", "Delta1block0": "1.0/(block0np1-1)",
                                    "Delta2block0": "2*M_PI/block0np2"}),
    # the TENO turbulent-channel app's discretisation: TENO6, power-law viscosity, constant
    # forcing, stretched wall-normal grid, SSP RK3 (the app's own parameters; its eps is the
    # generator's fixed 1e-40)
    "channel_tcf": ("channel_tcf", {"Re": "190.71", "gama": "1.4", "Minf": "0.0955", "Pr": "0.7", "Twall": "1.0",
                                    "dt": "0.0002", "niter": "10", "block0np0": "16", "block0np1": "17",
                                    "block0np2": "8", "Delta0block0": "4.0*M_PI/block0np0",
                                    "Delta1block0": "2.0/(block0np1-1)", "Delta2block0": "(4.0*M_PI/3.0)/block0np2",
                                    "c0": "-1", "c1": "0", "c2": "0", "stretch": "1.7", "TENO_CT": "1e-7",
                                    "eps": "1e-15"}),
    # Kelvin-Helmholtz with the classic SBLI RK3
    "kh_32": ("kh_weno5z", {"gama": "1.4", "dt": "0.0002", "niter": "6", "block0np0": "32", "block0np1": "32",
                            "Delta0block0": "1.0/block0np0", "Delta1block0": "1.0/block0np1", "khamp": "1.0",
                            "khphase": "0.0"}),
}


def plan_path(name):
    return os.path.join(HERE, "plan_%s.npz" % name)


def build_plan(name):
    """The BackendPlan GB300Backend derives from the reference's problem of case `name`."""
    import ref_generate
    case, params = CASES[name]
    block, _ = ref_generate.build_case(case)
    from opensbli import TraditionalAlgorithmRK
    from opensbli_gb300.backend import GB300Backend
    with open(os.devnull, "w") as dn, contextlib.redirect_stdout(dn):
        if hasattr(block, "nblocks"):  # a MultiBlock: the script's TraditionalAlgorithmRKMB
            from opensbli.multiblock.algorithm import TraditionalAlgorithmRKMB
            return GB300Backend(TraditionalAlgorithmRKMB(block), params, precision="fp64", blocks=block).plan()
        alg = TraditionalAlgorithmRK(block)
    return GB300Backend(alg, params, precision="fp64").plan()


def same_plan(a, b):
    """Whether two BackendPlans are identical (spec records, RK, dt, niter, arrays bit for bit)."""
    import numpy as np
    if (a.rk, a.dt, a.niter, a.precision, len(a.specs)) != (b.rk, b.dt, b.niter, b.precision, len(b.specs)):
        return False
    for ib in range(len(a.specs)):
        ra, xa = a.specs[ib].to_record()
        rb, xb = b.specs[ib].to_record()
        if ra != rb or sorted(xa) != sorted(xb) or any(not np.array_equal(xa[k], xb[k]) for k in xa):
            return False
        for ua, ub in ((a.states[ib], b.states[ib]), (a.coords[ib], b.coords[ib])):
            if (ua is None) != (ub is None):
                return False
            if ua is not None and (len(ua) != len(ub) or any(not np.array_equal(p, q) for p, q in zip(ua, ub))):
                return False
    return True


def main(argv):
    if argv and argv[0] == "--check":
        from opensbli_gb300.backend import BackendPlan
        ok = same_plan(build_plan(argv[1]), BackendPlan.load(plan_path(argv[1])))
        print("plan %s %s" % (argv[1], "unchanged" if ok else "CHANGED"))
        return 0 if ok else 1
    names = argv or sorted(CASES)
    for name in names:
        # one interpreter per case: the generator keeps module-level state between problems
        if len(names) > 1:
            import subprocess
            subprocess.check_call([sys.executable, os.path.abspath(__file__), name])
            continue
        plan = build_plan(name)
        plan.save(plan_path(name))
        print("wrote", plan_path(name), os.path.getsize(plan_path(name)), "bytes")
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv[1:]))
