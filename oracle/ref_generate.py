"""Generate the reference solver sources (OPS C++) for each parity case.

TEST INFRASTRUCTURE ONLY.  This script imports the upstream OpenSBLI generator from a
read-only checkout (``--reference``, default ``harness.reference_root()``), builds the problem
definitions below with OpenSBLI's own Python API, and writes the generated OPS C++
(``opensbli.cpp``, ``opensbliblock00_kernels.h``, ``defdec_data_set.h``, ...) into
``oracle/_ref/<case>/``.  Those sources are then compiled against ``oracle/ops_compat.h``
(``oracle/harness.py::build_ref``) and their output pins the C restatement in ``oracle/osb_oracle.c``.
Nothing under ``oracle/_ref`` is committed; it is regenerated from the reference.

The generator pins SymPy 1.1 (``environment_and_run_scripts/InstallPython.sh:50``); only
SymPy 1.14 exists here, so three runtime shims are applied (the checkout is not edited):

1. ``Indexed.is_commutative`` becomes a per-instance settable property
   (``opensbli/core/opensblifunctions.py:31`` assigns to it).
2. Bare integer ``0`` "equations" (zero entries of the eigenvector matrices,
   ``opensbli/schemes/spatial/shock_capturing.py:326-340``) are dropped before
   ``OPSC.kernel_computation_opsc`` (``opensbli/code_generation/opsc.py:629``).
3. ``GroupedPiecewise`` (``opensbli/core/opensbliobjects.py:672``) is printed as a C ternary
   through the printer's ``_print_Piecewise``.

Run parameters that OpenSBLI leaves as ``=Input`` are substituted by calls into
``ops_compat.h`` (``osb_env_int`` / ``osb_env_double``) so one compiled case can be run at
several sizes, time steps and step counts from the environment.
"""
import argparse
import os
import subprocess
import sys
import contextlib


HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(HERE))
import harness  # noqa: E402  (same directory: where the upstream checkout lies)


def apply_compat_patches():
    """The three SymPy-1.14 shims of the module docstring: the first is the package's front-end
    shim (opensbli_gb300.compat.apply, which a problem script run through GB300Backend needs
    too), the other two concern only the OPS printer."""
    import sympy
    from opensbli_gb300 import compat
    compat.apply()

    from opensbli.code_generation import opsc as opsc_mod
    from opensbli.core.opensbliobjects import GroupedPiecewise

    orig_kc = opsc_mod.OPSC.kernel_computation_opsc

    def kernel_computation_opsc(self, kernel):
        kernel.equations = [e for e in kernel.equations
                            if not (isinstance(e, int) or (hasattr(e, "is_zero") and e is sympy.S.Zero))]
        return orig_kc(self, kernel)

    opsc_mod.OPSC.kernel_computation_opsc = kernel_computation_opsc

    printer = opsc_mod.OPSCCodePrinter

    def _print_GroupedPiecewise(self, expr):
        return printer._print_Piecewise(self, sympy.Piecewise(*expr.args))

    printer._print_GroupedPiecewise = _print_GroupedPiecewise


@contextlib.contextmanager
def in_dir(path):
    old = os.getcwd()
    os.makedirs(path, exist_ok=True)
    os.chdir(path)
    try:
        yield
    finally:
        os.chdir(old)


def _env_params(ndim, defaults):
    """Map OpenSBLI ``Input`` constants to environment-driven C expressions."""
    names, values = [], []
    for k, v in defaults.items():
        names.append(k)
        values.append(v)
    return names, values


def _euler_equations(ndim, scheme_tag, viscous=False):
    """Conservative Euler / Navier-Stokes equations in OpenSBLI's Einstein notation
    (the forms of ``apps/compressible_taylor_green_vortex/compressible_TGV.py:43-59``)."""
    from opensbli import EinsteinEquation, SimulationEquations
    sc1 = "**{'scheme':'%s'}" % scheme_tag
    constants = ["Re", "Pr", "gama", "Minf", "SuthT", "RefT"]
    eq = EinsteinEquation()
    mass = "Eq(Der(rho,t), - Conservative(rhou_j,x_j,%s))" % sc1
    if viscous:
        momentum = "Eq(Der(rhou_i,t) , -Conservative(rhou_i*u_j + KD(_i,_j)*p,x_j , %s) + Der(tau_i_j,x_j) )" % sc1
        energy = "Eq(Der(rhoE,t), - Conservative((p+rhoE)*u_j,x_j, %s) - Der(q_j,x_j) + Der(u_i*tau_i_j ,x_j) )" % sc1
        subs = ["Eq(tau_i_j, (mu/Re)*(Der(u_i,x_j)+ Der(u_j,x_i) - (2/3)* KD(_i,_j)* Der(u_k,x_k)))",
                "Eq(q_j, (-mu/((gama-1)*Minf*Minf*Pr*Re))*Der(T,x_j))"]
    else:
        momentum = "Eq(Der(rhou_i,t) , -Conservative(rhou_i*u_j + KD(_i,_j)*p,x_j , %s))" % sc1
        energy = "Eq(Der(rhoE,t), - Conservative((p+rhoE)*u_j,x_j, %s))" % sc1
        subs = []
    sim = SimulationEquations()
    for base in (mass, momentum, energy):
        sim.add_equations(eq.expand(base, ndim, "x", subs, constants))
    return sim


def _constituents(ndim, viscous=False, sutherland=True, with_T=None):
    from opensbli import EinsteinEquation, ConstituentRelations
    eq = EinsteinEquation()
    constants = ["Re", "Pr", "gama", "Minf", "SuthT", "RefT"]
    rels = ["Eq(u_i, rhou_i/rho)",
            "Eq(p, (gama-1)*(rhoE - (1/2)*rho*(KD(_i,_j)*u_i*u_j)))"]
    if viscous or with_T:
        rels.append("Eq(T, p*gama*Minf*Minf/(rho))")
    rels.append("Eq(H, (rhoE + p) / rho)")
    if viscous and sutherland:
        rels.append("Eq(mu, (T**(1.5)*(1.4042)/(T+0.40417)))")
    rels.append("Eq(a, (gama*p/rho)**0.5)")
    cr = ConstituentRelations()
    for r in rels:
        cr.add_equations(eq.expand(r, ndim, "x", [], constants))
    return cr


def _finish(block, alg_kwargs, params):
    from opensbli import TraditionalAlgorithmRK, SimulationDataType, Double, OPSC
    from opensbli.utilities.helperfunctions import substitute_simulation_parameters
    if hasattr(block, "nblocks"):  # a MultiBlock: the multi-block time loop (multiblock/algorithm.py)
        from opensbli.multiblock.algorithm import TraditionalAlgorithmRKMB
        alg = TraditionalAlgorithmRKMB(block, **alg_kwargs)
    else:
        alg = TraditionalAlgorithmRK(block, **alg_kwargs)
    SimulationDataType.set_datatype(Double)
    OPSC(alg)
    names, values = zip(*params.items())
    substitute_simulation_parameters(list(names), list(values))


def case_sod_extrap():
    """1D Sod as case_sod_weno5js but with extrapolation boundaries: linear (order 1) on the
    left, zeroth order on the right (core/boundary_conditions/extrapolation.py)."""
    from opensbli import ExtrapolationBC
    block, params = case_sod_weno5js(bcs=[ExtrapolationBC(0, 0, order=1), ExtrapolationBC(0, 1, order=0)])
    return block, params


def case_sod_weno5js(bcs=None):
    """1D Sod, WENO5-JS characteristic LLF (simple average), zero-gradient ends, RK-LS3.
    Problem definition follows ``apps/Sod_shock_tube/Sod_shock_tube.py`` with the
    scheme/BC/time-stepper choices of the 1D Sod parity case."""
    import copy
    from opensbli import (SimulationBlock, GridBasedInitialisation, GridVariable, DataObject,
                          parse_expr, SimpleAverage, LFWeno, RungeKuttaLS, ZeroGradientOutletBC)
    ndim = 1
    sim = _euler_equations(ndim, "Weno")
    cr = _constituents(ndim)
    block = SimulationBlock(ndim, block_number=0)
    local_dict = {"block": block, "GridVariable": GridVariable, "DataObject": DataObject}
    eqns = ["Eq(DataObject(x0), block.deltas[0]*block.grid_indexes[0])",
            "Eq(GridVariable(u0), Piecewise((0.0, DataObject(x0) < 0.5),(0, True)))",
            "Eq(GridVariable(p), Piecewise((1.0, DataObject(x0) < 0.5), (0.10, True)))",
            "Eq(GridVariable(d), Piecewise((1.0, DataObject(x0) < 0.5), (0.125, True)))",
            "Eq(DataObject(rho), d)", "Eq(DataObject(rhou0), d*u0)",
            "Eq(DataObject(rhoE), p/(gama-1.0) + 0.5* d *(u0**2.0))"]
    initial = GridBasedInitialisation()
    initial.add_equations([parse_expr(e, local_dict=local_dict) for e in eqns])
    schemes = {}
    LF = LFWeno(order=5, formulation="JS", averaging=SimpleAverage([0, 1]), flux_type="LLF")
    schemes[LF.name] = LF
    rk = RungeKuttaLS(3)
    schemes[rk.name] = rk
    block.set_block_boundaries(bcs or [ZeroGradientOutletBC(0, 0), ZeroGradientOutletBC(0, 1)])
    block.set_equations([copy.deepcopy(cr), copy.deepcopy(sim), initial])
    block.set_discretisation_schemes(schemes)
    block.discretise()
    params = {"gama": "1.4", "dt": 'osb_env_double("OSB_DT", 0.0002)',
              "niter": 'osb_env_int("OSB_NITER", 1)', "block0np0": 'osb_env_int("OSB_NP0", 400)',
              "Delta0block0": "1.0/(block0np0-1)"}
    return block, params


def _tgv_block(ndim, conservative=True):
    from opensbli import SimulationBlock, GridBasedInitialisation, GridVariable, DataObject, parse_expr
    block = SimulationBlock(ndim, block_number=0, conservative=conservative)
    local_dict = {"block": block, "GridVariable": GridVariable, "DataObject": DataObject}
    eqns = ["Eq(GridVariable(x0), block.deltas[0]*block.grid_indexes[0])",
            "Eq(GridVariable(x1), block.deltas[1]*block.grid_indexes[1])",
            "Eq(GridVariable(x2), block.deltas[2]*block.grid_indexes[2])",
            "Eq(GridVariable(u0),sin(x0)*cos(x1)*cos(x2))",
            "Eq(GridVariable(u1),-cos(x0)*sin(x1)*cos(x2))",
            "Eq(GridVariable(u2), 0.0)",
            "Eq(GridVariable(p), 1.0/(gama*Minf*Minf)+ (1.0/16.0) * (cos(2.0*x0)+cos(2.0*x1))*(2.0 + cos(2.0*x2)))",
            "Eq(GridVariable(r), gama*Minf*Minf*p)",
            "Eq(DataObject(rho), r)", "Eq(DataObject(rhou0), r*u0)", "Eq(DataObject(rhou1), r*u1)",
            "Eq(DataObject(rhou2), r*u2)",
            "Eq(DataObject(rhoE), p/(gama-1) + 0.5* r *(u0**2+ u1**2 + u2**2))"]
    initial = GridBasedInitialisation()
    initial.add_equations([parse_expr(e, local_dict=local_dict) for e in eqns])
    return block, initial


def _tgv_params(minf, n, dt):
    p = {"Re": "1600.0", "gama": "1.4", "Minf": str(minf), "Pr": "0.71",
         "dt": 'osb_env_double("OSB_DT", %s)' % dt, "niter": 'osb_env_int("OSB_NITER", 1)'}
    for d in range(3):
        p["block0np%d" % d] = 'osb_env_int("OSB_NP%d", %d)' % (d, n)
        p["Delta%dblock0" % d] = "2*M_PI/block0np%d" % d
    p["TENO_CT"] = 'osb_env_double("OSB_TENO_CT", 1e-6)'
    return p


def case_tgv_shock(kind):
    """3D supersonic TGV: characteristic LLF TENO5 (Roe average) or WENO5-Z (simple average)
    plus 4th-order central viscous terms (StoreSome), periodic, RK-LS3
    (``apps/compressible_taylor_green_vortex/compressible_TGV.py:43-242``)."""
    import copy
    from opensbli import (SimpleAverage, RoeAverage, LFWeno, LFTeno, StoreSome, RungeKuttaLS, PeriodicBC)
    ndim = 3
    tag = "Teno" if kind.startswith("teno") else "Weno"
    sim = _euler_equations(ndim, tag, viscous=True)
    cr = _constituents(ndim, viscous=True)
    block, initial = _tgv_block(ndim)
    schemes = {}
    if kind == "teno5":
        LF = LFTeno(order=5, averaging=RoeAverage([0, 1]), flux_type="LLF")
    elif kind == "teno6":
        LF = LFTeno(order=6, averaging=RoeAverage([0, 1]), flux_type="LLF")
    else:
        LF = LFWeno(order=5, formulation="Z", averaging=SimpleAverage([0, 1]), flux_type="LLF")
    schemes[LF.name] = LF
    cent = StoreSome(4, "u0 u1 u2")
    schemes[cent.name] = cent
    rk = RungeKuttaLS(3)
    schemes[rk.name] = rk
    block.set_discretisation_schemes(schemes)
    bcs = []
    for d in range(ndim):
        bcs += [PeriodicBC(d, 0, halos=[-4, 4]), PeriodicBC(d, 1, halos=[-4, 4])]
    block.set_block_boundaries(bcs)
    block.set_equations([copy.deepcopy(cr), copy.deepcopy(sim), initial])
    block.discretise()
    return block, _tgv_params(1.25, 16, "0.001")


def case_tgv_central():
    """3D low-Mach TGV, 4th-order central Feiereisen split form with constant viscosity,
    periodic, RK-LS3 (``apps/taylor_green_vortex/taylor_green_vortex.py:20-140``; no DRP filter)."""
    import copy
    from opensbli import (NS_Split, SimulationEquations, ConstituentRelations, EinsteinEquation,
                          StoreSome, RungeKuttaLS, PeriodicBC)
    ndim = 3
    constants = ["Re", "Pr", "gama", "Minf", "mu"]
    NS = NS_Split("Feiereisen", ndim, constants, coordinate_symbol="x", conservative=True,
                  viscosity="constant")
    sim = SimulationEquations()
    sim.add_equations(NS.mass)
    sim.add_equations(NS.momentum)
    sim.add_equations(NS.energy)
    cr = ConstituentRelations()
    ee = EinsteinEquation()
    for r in ["Eq(u_i, rhou_i/rho)", "Eq(p, (gama-1)*(rhoE - (1/2)*rho*(KD(_i,_j)*u_i*u_j)))",
              "Eq(T, p*gama*Minf*Minf/(rho))"]:
        cr.add_equations(ee.expand(r, ndim, "x", [], constants))
    block, initial = _tgv_block(ndim)
    schemes = {}
    cent = StoreSome(4, "u0 u1 u2")
    schemes[cent.name] = cent
    rk = RungeKuttaLS(3)
    schemes[rk.name] = rk
    block.set_discretisation_schemes(schemes)
    bcs = []
    for d in range(ndim):
        bcs += [PeriodicBC(d, 0, full_depth=True), PeriodicBC(d, 1, full_depth=True)]
    block.set_block_boundaries(bcs)
    block.set_equations([copy.deepcopy(cr), copy.deepcopy(sim), initial])
    block.discretise()
    return block, _tgv_params(0.1, 16, "0.003385")


def central_split_block(form, energy_formulation="none", extra=None):
    """3D supersonic TGV block with the central 4th-order scheme and the convective split form
    `form` of physical_models/split_forms.py (NS_Split), modified Sutherland viscosity
    (StoreSome), RK-LS3, periodic -- the central branch of
    ``apps/compressible_taylor_green_vortex/compressible_TGV.py:66-75, 128-160``.  extra(block),
    when given, adds a filter's equation classes before discretisation and returns the filter,
    whose periodic exchange of depth 4 is then added after it (that app's lines 210-222)."""
    import copy
    from opensbli import NS_Split, SimulationEquations, StoreSome, RungeKuttaLS, PeriodicBC
    ndim = 3
    constants = ["Re", "Pr", "gama", "Minf", "SuthT", "RefT"]
    NS = NS_Split(form, ndim, constants, coordinate_symbol="x", conservative=True, viscosity="dynamic",
                  energy_formulation=energy_formulation, debug=False)
    sim = SimulationEquations()
    sim.add_equations(NS.mass)
    sim.add_equations(NS.momentum)
    sim.add_equations(NS.energy)
    cr = _constituents(ndim, viscous=True)
    block, initial = _tgv_block(ndim)
    schemes = {}
    cent = StoreSome(4, "u0 u1 u2")
    schemes[cent.name] = cent
    rk = RungeKuttaLS(3)
    schemes[rk.name] = rk
    block.set_discretisation_schemes(schemes)
    bcs = []
    for d in range(ndim):
        bcs += [PeriodicBC(d, 0, halos=[-2, 2]), PeriodicBC(d, 1, halos=[-2, 2])]
    block.set_block_boundaries(bcs)
    block.set_equations([copy.deepcopy(cr), copy.deepcopy(sim), initial])
    filt = extra(block) if extra else None
    block.discretise()
    if filt is not None:
        filt.update_periodic_boundary(block, halos=[-4, 4])
    return block, _tgv_params(1.25, 16, "0.001")


def case_channel_adi():
    """The channel of case_channel_iso with the upper wall adiabatic (AdiabaticWallBC, the
    alternative upper wall of ``apps/channel_flow/laminar_2D/laminar_channel.py:104-113``)."""
    return case_channel_iso(upper="adiabatic")


def case_channel_iso(upper="isothermal", stretch=False):
    """3D channel between isothermal no-slip walls: characteristic LLF TENO5 (Roe average) plus
    4th-order central viscous terms (StoreSome), the shock-capturing form of the SBLI apps, on a
    uniform grid; IsothermalWallBC on both y faces with the wall energy of
    ``apps/channel_flow/compressible_TCF_Central/turbulent_channel.py:118-131`` (no forcing
    terms), periodic in x and z, RK-LS3.  The wall faces take the reference's default Carpenter
    closures of the central derivatives (core/boundary_conditions/Carpenter_scheme.py).

    stretch=True: the wall-normal grid of ``apps/channel_flow/compressible_TCF_TENO/
    turbulent_channel.py:170-232``, x1 = -tanh(stretch (1 - 2 j / (N_y - 1))) / tanh(stretch) with
    stretch = 1.7 on xi_1 in [0, 1] (Delta_1 = 1 / (N_y - 1)), transformed by a MetricsEquation
    with direction 1 stretched only and applied to the equations (``apply_metrics``); the
    velocity, pressure and density fields take the grid's x0, x1, x2."""
    import copy
    from opensbli import (RoeAverage, LFTeno, StoreSome, RungeKuttaLS, PeriodicBC, IsothermalWallBC,
                          AdiabaticWallBC, SimulationBlock, GridBasedInitialisation, GridVariable, DataObject,
                          parse_expr, ConstantObject, Eq, MetricsEquation)
    ndim = 3
    sim = _euler_equations(ndim, "Teno", viscous=True)
    cr = _constituents(ndim, viscous=True)
    block = SimulationBlock(ndim, block_number=0)
    local_dict = {"block": block, "GridVariable": GridVariable, "DataObject": DataObject}
    fields = ["Eq(GridVariable(u0), (1.0 - x1*x1)*(1.0 + 0.1*sin(x0)*cos(x2)))",
              "Eq(GridVariable(u1), 0.05*sin(x0)*(1.0 - x1*x1)*(1.0 - x1*x1))",
              "Eq(GridVariable(u2), 0.05*cos(x0)*sin(x2)*(1.0 - x1*x1))",
              "Eq(GridVariable(p), 1.0/(gama*Minf*Minf)*(1.0 + 0.02*cos(x0)*cos(x2)))",
              "Eq(GridVariable(r), 1.0 + 0.02*sin(x0)*x1)",
              "Eq(DataObject(rho), r)", "Eq(DataObject(rhou0), r*u0)", "Eq(DataObject(rhou1), r*u1)",
              "Eq(DataObject(rhou2), r*u2)",
              "Eq(DataObject(rhoE), p/(gama-1) + 0.5* r *(u0**2+ u1**2 + u2**2))"]
    initial = GridBasedInitialisation()
    if stretch:
        from sympy import tanh
        (i, j, k) = block.grid_indexes
        (dx, dy, dz) = block.deltas
        ny, st = ConstantObject("block0np1"), ConstantObject("stretch")
        x1 = 0.5 * 2 * (1.0 - tanh(st * (1.0 - 2.0 * (j / (ny - 1.0)))) / tanh(st)) - 1.0
        grid = [Eq(DataObject("x0"), i * dx), Eq(DataObject("x1"), x1), Eq(DataObject("x2"), k * dz)]
        fields = [f.replace("x0", "DataObject(x0)").replace("x1", "DataObject(x1)").replace("x2", "DataObject(x2)")
                  for f in fields]
        initial.add_equations(grid + [parse_expr(e, local_dict=local_dict) for e in fields])
        metriceq = MetricsEquation()
        metriceq.generate_transformations(ndim, "x", [(False, False), (True, False), (False, False)], 2)
        sim.apply_metrics(metriceq)
        equations = [copy.deepcopy(cr), sim, initial, metriceq]
    else:
        eqns = ["Eq(GridVariable(x0), block.deltas[0]*block.grid_indexes[0])",
                "Eq(GridVariable(x1), -1.0 + block.deltas[1]*block.grid_indexes[1])",
                "Eq(GridVariable(x2), block.deltas[2]*block.grid_indexes[2])"] + fields
        initial.add_equations([parse_expr(e, local_dict=local_dict) for e in eqns])
        equations = [copy.deepcopy(cr), copy.deepcopy(sim), initial]
    schemes = {}
    LF = LFTeno(order=5, averaging=RoeAverage([0, 1]), flux_type="LLF")
    schemes[LF.name] = LF
    cent = StoreSome(4, "u0 u1 u2 T" if stretch else "u0 u1 u2")
    schemes[cent.name] = cent
    rk = RungeKuttaLS(3)
    schemes[rk.name] = rk
    block.set_discretisation_schemes(schemes)
    q = flatten_q(sim)
    gama, Minf, Twall = ConstantObject("gama"), ConstantObject("Minf"), ConstantObject("Twall")
    wall = [Eq(q[4], Twall * q[0] / (gama * Minf ** 2.0 * (gama - 1)))]
    bcs = [PeriodicBC(0, 0, halos=[-4, 4]), PeriodicBC(0, 1, halos=[-4, 4]),
           IsothermalWallBC(1, 0, wall[:]),
           IsothermalWallBC(1, 1, wall[:]) if upper == "isothermal" else AdiabaticWallBC(1, 1),
           PeriodicBC(2, 0, halos=[-4, 4]), PeriodicBC(2, 1, halos=[-4, 4])]
    block.set_block_boundaries(bcs)
    block.set_equations(equations)
    block.discretise()
    p = {"Re": "100.0", "gama": "1.4", "Minf": "0.5", "Pr": "0.71", "Twall": "1.0",
         "dt": 'osb_env_double("OSB_DT", 0.001)', "niter": 'osb_env_int("OSB_NITER", 1)',
         "TENO_CT": 'osb_env_double("OSB_TENO_CT", 1e-6)'}
    if stretch:
        p["stretch"] = "1.7"
    d1 = "1.0/(block0np1-1)" if stretch else "2.0/(block0np1-1)"
    for d, (n, dl) in enumerate([(16, "2*M_PI/block0np0"), (17, d1), (8, "2*M_PI/block0np2")]):
        p["block0np%d" % d] = 'osb_env_int("OSB_NP%d", %d)' % (d, n)
        p["Delta%dblock0" % d] = dl
    return block, p


def case_channel_tcf():
    """The equations and schemes of ``apps/channel_flow/compressible_TCF_TENO/turbulent_channel.py``
    (lines 35-93, 139-246): Navier-Stokes with the constant forcing terms -KD(_i,_j) c_j and
    -Dot(c_j, u_j), power-law viscosity mu = T^0.7, characteristic LLF TENO6 (Roe average),
    StoreSome(4, 'u0 u1 u2 T'), the SSP RK3, isothermal walls on both y faces (Twall), periodic x
    and z, and the tanh-stretched wall-normal grid on xi_1 in [0, 2] transformed by a
    MetricsEquation stretched in y; the app's parameters (Re 190.71, Minf 0.0955, Pr 0.7,
    c = (-1, 0, 0), stretch 1.7, TENO_CT 1e-7, eps 1e-15) on a 16 x 17 x 8 block.  The
    initial fields are the channel cases' (the golden runs replace them); the statistics
    classes and the HDF5 output of the app are not part of the residual path."""
    import copy
    from sympy import tanh
    from opensbli import (EinsteinEquation, SimulationEquations, ConstituentRelations, RoeAverage, LFTeno,
                          StoreSome, RungeKuttaLS, PeriodicBC, IsothermalWallBC, SimulationBlock,
                          GridBasedInitialisation, GridVariable, DataObject, parse_expr, ConstantObject, Eq,
                          MetricsEquation)
    ndim = 3
    sc1 = "**{'scheme':'Teno'}"
    mass = "Eq(Der(rho,t), - Conservative(rhou_j,x_j,%s))" % sc1
    momentum = ("Eq(Der(rhou_i,t) , -Conservative(rhou_i*u_j + KD(_i,_j)*p,x_j , %s) + Der(tau_i_j,x_j) "
                "- KD(_i,_j)*c_j )" % sc1)
    energy = ("Eq(Der(rhoE,t), - Conservative((p+rhoE)*u_j,x_j, %s) - Der(q_j,x_j) + Der(u_i*tau_i_j ,x_j) "
              "- Dot(c_j, u_j))" % sc1)
    subs = ["Eq(tau_i_j, (mu/Re)*(Der(u_i,x_j)+ Der(u_j,x_i) - (2/3)* KD(_i,_j)* Der(u_k,x_k)))",
            "Eq(q_j, (-mu/((gama-1)*Minf*Minf*Pr*Re))*Der(T,x_j))"]
    constants = ["Re", "Pr", "gama", "Minf", "c_j"]
    eq = EinsteinEquation()
    sim = SimulationEquations()
    for base in (mass, momentum, energy):
        sim.add_equations(eq.expand(base, ndim, "x", subs, constants))
    cr = ConstituentRelations()
    for r in ["Eq(u_i, rhou_i/rho)", "Eq(p, (gama-1)*(rhoE - rho*(1/2)*(KD(_i,_j)*u_i*u_j)))",
              "Eq(a, (gama*p/rho)**0.5)", "Eq(T, p*gama*Minf*Minf/(rho))", "Eq(mu, (T**0.7))"]:
        cr.add_equations(eq.expand(r, ndim, "x", subs, constants))
    block = SimulationBlock(ndim, block_number=0)
    local_dict = {"block": block, "GridVariable": GridVariable, "DataObject": DataObject}
    (i, j, k) = block.grid_indexes
    (dx, dy, dz) = block.deltas
    ny, st = ConstantObject("block0np1"), ConstantObject("stretch")
    x1 = 0.5 * 2 * (1.0 - tanh(st * (1.0 - 2.0 * (j / (ny - 1.0)))) / tanh(st)) - 1.0
    grid = [Eq(DataObject("x0"), i * dx), Eq(DataObject("x1"), x1), Eq(DataObject("x2"), k * dz)]
    fields = ["Eq(GridVariable(u0), (1.0 - DataObject(x1)*DataObject(x1))*(1.0 + 0.1*sin(DataObject(x0))*cos(DataObject(x2))))",
              "Eq(GridVariable(u1), 0.05*sin(DataObject(x0))*(1.0 - DataObject(x1)*DataObject(x1))*(1.0 - DataObject(x1)*DataObject(x1)))",
              "Eq(GridVariable(u2), 0.05*cos(DataObject(x0))*sin(DataObject(x2))*(1.0 - DataObject(x1)*DataObject(x1)))",
              "Eq(GridVariable(p), 1.0/(gama*Minf*Minf)*(1.0 + 0.02*cos(DataObject(x0))*cos(DataObject(x2))))",
              "Eq(GridVariable(r), 1.0 + 0.02*sin(DataObject(x0))*DataObject(x1))",
              "Eq(DataObject(rho), r)", "Eq(DataObject(rhou0), r*u0)", "Eq(DataObject(rhou1), r*u1)",
              "Eq(DataObject(rhou2), r*u2)",
              "Eq(DataObject(rhoE), p/(gama-1) + 0.5* r *(u0**2+ u1**2 + u2**2))"]
    initial = GridBasedInitialisation()
    initial.add_equations(grid + [parse_expr(e, local_dict=local_dict) for e in fields])
    metriceq = MetricsEquation()
    metriceq.generate_transformations(ndim, "x", [(False, False), (True, False), (False, False)], 2)
    sim.apply_metrics(metriceq)
    schemes = {}
    LF = LFTeno(order=6, averaging=RoeAverage([0, 1]), flux_type="LLF")
    schemes[LF.name] = LF
    cent = StoreSome(4, "u0 u1 u2 T")
    schemes[cent.name] = cent
    rk = RungeKuttaLS(3, formulation="SSP")
    schemes[rk.name] = rk
    block.set_discretisation_schemes(schemes)
    q = flatten_q(sim)
    gama, Minf, Twall = ConstantObject("gama"), ConstantObject("Minf"), ConstantObject("Twall")
    wall = [Eq(q[4], Twall * q[0] / (gama * Minf ** 2.0 * (gama - 1)))]
    bcs = [PeriodicBC(0, 0), PeriodicBC(0, 1), IsothermalWallBC(1, 0, wall[:]), IsothermalWallBC(1, 1, wall[:]),
           PeriodicBC(2, 0), PeriodicBC(2, 1)]
    block.set_block_boundaries(bcs)
    block.set_equations([copy.deepcopy(cr), sim, initial, metriceq])
    block.discretise()
    p = {"Re": "190.71", "gama": "1.4", "Minf": "0.0955", "Pr": "0.7", "Twall": "1.0", "stretch": "1.7",
         "c0": "-1", "c1": "0", "c2": "0", "eps": "1e-15",
         "dt": 'osb_env_double("OSB_DT", 0.0002)', "niter": 'osb_env_int("OSB_NITER", 1)',
         "TENO_CT": 'osb_env_double("OSB_TENO_CT", 1e-7)'}
    for d, (n, dl) in enumerate([(16, "4.0*M_PI/block0np0"), (17, "2.0/(block0np1-1)"), (8, "(4.0*M_PI/3.0)/block0np2")]):
        p["block0np%d" % d] = 'osb_env_int("OSB_NP%d", %d)' % (d, n)
        p["Delta%dblock0" % d] = dl
    return block, p


def case_duct_inlet(minf=0.5):
    """The inflow / outflow faces of the SBLI apps (apps/katzer_SBLI/katzer_SBLI.py:131-160) on a
    3D duct: InletPressureExtrapolateBC at x = 0 and ExtrapolationBC(order=0) at the far x face,
    isothermal no-slip walls on both y faces, periodic z; characteristic LLF TENO5 (Roe average)
    plus central viscous terms, RK-LS3, Minf = `minf` (0.5: the subsonic branch of the inlet, the
    pressure extrapolated into its halos; 2: the supersonic branch).  The inlet, outlet and wall
    faces are ModifyCentralDerivative boundaries: the viscous terms take the Carpenter closures
    at all four.  The inflow state is what the initialisation left in the inlet's halos."""
    import copy
    from opensbli import (RoeAverage, LFTeno, StoreSome, RungeKuttaLS, PeriodicBC, IsothermalWallBC,
                          SimulationBlock, GridBasedInitialisation, GridVariable, DataObject, parse_expr,
                          ConstantObject, Eq)
    from opensbli.core.boundary_conditions.inlet_pressure_extrapolate import InletPressureExtrapolateBC
    from opensbli.core.boundary_conditions.extrapolation import ExtrapolationBC
    ndim = 3
    sim = _euler_equations(ndim, "Teno", viscous=True)
    cr = _constituents(ndim, viscous=True)
    block = SimulationBlock(ndim, block_number=0)
    local_dict = {"block": block, "GridVariable": GridVariable, "DataObject": DataObject}
    eqns = ["Eq(GridVariable(x0), block.deltas[0]*block.grid_indexes[0])",
            "Eq(GridVariable(x1), -1.0 + block.deltas[1]*block.grid_indexes[1])",
            "Eq(GridVariable(x2), block.deltas[2]*block.grid_indexes[2])",
            "Eq(GridVariable(u0), (1.0 - x1*x1)*(1.0 + 0.05*sin(x2)))",
            "Eq(GridVariable(u1), 0.05*sin(x0)*(1.0 - x1*x1)*(1.0 - x1*x1))",
            "Eq(GridVariable(u2), 0.05*cos(x0)*sin(x2)*(1.0 - x1*x1))",
            "Eq(GridVariable(p), 1.0/(gama*Minf*Minf)*(1.0 + 0.02*cos(x0)*cos(x2)))",
            "Eq(GridVariable(r), 1.0 + 0.02*sin(x0)*x1)",
            "Eq(DataObject(rho), r)", "Eq(DataObject(rhou0), r*u0)", "Eq(DataObject(rhou1), r*u1)",
            "Eq(DataObject(rhou2), r*u2)",
            "Eq(DataObject(rhoE), p/(gama-1) + 0.5* r *(u0**2+ u1**2 + u2**2))"]
    initial = GridBasedInitialisation()
    initial.add_equations([parse_expr(e, local_dict=local_dict) for e in eqns])
    schemes = {}
    LF = LFTeno(order=5, averaging=RoeAverage([0, 1]), flux_type="LLF")
    schemes[LF.name] = LF
    cent = StoreSome(4, "u0 u1 u2")
    schemes[cent.name] = cent
    rk = RungeKuttaLS(3)
    schemes[rk.name] = rk
    block.set_discretisation_schemes(schemes)
    q = flatten_q(sim)
    gama, Minf, Twall = ConstantObject("gama"), ConstantObject("Minf"), ConstantObject("Twall")
    wall = [Eq(q[4], Twall * q[0] / (gama * Minf ** 2.0 * (gama - 1)))]
    bcs = [InletPressureExtrapolateBC(0, 0), ExtrapolationBC(0, 1, order=0),
           IsothermalWallBC(1, 0, wall[:]), IsothermalWallBC(1, 1, wall[:]),
           PeriodicBC(2, 0, halos=[-4, 4]), PeriodicBC(2, 1, halos=[-4, 4])]
    block.set_block_boundaries(bcs)
    block.set_equations([copy.deepcopy(cr), copy.deepcopy(sim), initial])
    block.discretise()
    p = {"Re": "100.0", "gama": "1.4", "Minf": repr(float(minf)), "Pr": "0.71", "Twall": "1.0",
         "dt": 'osb_env_double("OSB_DT", 0.0005)', "niter": 'osb_env_int("OSB_NITER", 1)',
         "TENO_CT": 'osb_env_double("OSB_TENO_CT", 1e-6)'}
    for d, (n, dl) in enumerate([(20, "4.0/(block0np0-1)"), (17, "2.0/(block0np1-1)"), (8, "2*M_PI/block0np2")]):
        p["block0np%d" % d] = 'osb_env_int("OSB_NP%d", %d)' % (d, n)
        p["Delta%dblock0" % d] = dl
    return block, p


def case_katzer():
    """The discretisation of ``apps/katzer_SBLI/katzer_SBLI.py`` (its direct shock-capturing
    branch, lines 30-160): 2D Navier-Stokes with WENO5-Z (simple average, LLF), StoreSome(4,
    'u0 u1 T'), the Sutherland law mu = T^1.5 (1 + SuthT/RefT) / (T + SuthT/RefT), the SSP RK3, a
    sinh-stretched wall-normal grid (Lx1 sinh(by xi_1 / Lx1) / sinh(by)) transformed by a
    MetricsEquation stretched in y, the pressure-extrapolation inlet at x = 0, zeroth-order
    extrapolation at the far x face, an isothermal wall (Twall 1.67619431) at y = 0 and the app's
    Dirichlet shock-generator state at the top (post-shock where x0 > 40); the app's parameters
    (Minf 2, Re 950, Pr 0.72) on a 24 x 17 block.  The app's similarity-solution initialisation
    (Initialise_Katzer) is replaced by analytic fields: the golden runs replace the state anyway."""
    import copy
    from sympy import sinh
    from opensbli import (EinsteinEquation, SimulationEquations, ConstituentRelations, SimpleAverage, LFWeno,
                          StoreSome, RungeKuttaLS, IsothermalWallBC, DirichletBC, SimulationBlock,
                          GridBasedInitialisation, GridVariable, DataObject, parse_expr, ConstantObject, Eq,
                          MetricsEquation)
    from opensbli.core.boundary_conditions.inlet_pressure_extrapolate import InletPressureExtrapolateBC
    from opensbli.core.boundary_conditions.extrapolation import ExtrapolationBC
    ndim = 2
    eq = EinsteinEquation()
    constants = ["Re", "Pr", "gama", "Minf", "SuthT", "RefT"]
    sc1 = "**{'scheme':'Weno'}"
    mass = "Eq(Der(rho,t), - Conservative(rhou_j,x_j,%s))" % sc1
    momentum = "Eq(Der(rhou_i,t) , -Conservative(rhou_i*u_j + KD(_i,_j)*p,x_j , %s) + Der(tau_i_j,x_j) )" % sc1
    energy = "Eq(Der(rhoE,t), - Conservative((p+rhoE)*u_j,x_j, %s) - Der(q_j,x_j) + Der(u_i*tau_i_j ,x_j) )" % sc1
    subs = ["Eq(tau_i_j, (mu/Re)*(Der(u_i,x_j)+ Der(u_j,x_i) - (2/3)* KD(_i,_j)* Der(u_k,x_k)))",
            "Eq(q_j, (-mu/((gama-1)*Minf*Minf*Pr*Re))*Der(T,x_j))"]
    sim = SimulationEquations()
    for base in (mass, momentum, energy):
        sim.add_equations(eq.expand(base, ndim, "x", subs, constants))
    cr = ConstituentRelations()
    for r in ["Eq(u_i, rhou_i/rho)", "Eq(p, (gama-1)*(rhoE - rho*(1/2)*(KD(_i,_j)*u_i*u_j)))",
              "Eq(a, (gama*p/rho)**0.5)", "Eq(T, p*gama*Minf*Minf/(rho))",
              "Eq(mu, (T**(1.5)*(1.0+SuthT/RefT)/(T+SuthT/RefT)))"]:
        cr.add_equations(eq.expand(r, ndim, "x", [], constants))
    block = SimulationBlock(ndim, block_number=0)
    metriceq = MetricsEquation()
    metriceq.generate_transformations(ndim, "x", [(False, False), (True, False)], 2)
    sim.apply_metrics(metriceq)
    schemes = {}
    LF = LFWeno(order=5, formulation="Z", averaging=SimpleAverage([0, 1]), flux_type="LLF")
    schemes[LF.name] = LF
    cent = StoreSome(4, "u0 u1 T")
    schemes[cent.name] = cent
    rk = RungeKuttaLS(3, formulation="SSP")
    schemes[rk.name] = rk
    block.set_discretisation_schemes(schemes)
    local_dict = {"block": block, "GridVariable": GridVariable, "DataObject": DataObject}
    for con in ["Minf", "Twall", "Lx1", "by"]:
        local_dict[con] = ConstantObject(con)
    x_loc = parse_expr("Eq(GridVariable(x0), block.deltas[0]*block.grid_indexes[0])", local_dict=local_dict)
    q = flatten_q(sim)
    rhoE_wall = parse_expr("Eq(DataObject(rhoE), DataObject(rho)*Twall/(gama*(gama-1.0)*Minf**2.0))",
                           local_dict=local_dict)
    top = [parse_expr(e, local_dict=local_dict) for e in [
        "Eq(DataObject(rho), Piecewise((1.129734572, (x0)>40.0), (1.00000596004, True)))",
        "Eq(DataObject(rhou0), Piecewise((1.0921171, (x0)>40.0), (1.00000268202, True)))",
        "Eq(DataObject(rhou1), Piecewise((-0.058866065, (x0)>40.0), (0.00565001630205, True)))",
        "Eq(DataObject(rhoE), Piecewise((1.0590824, (x0)>40.0), (0.94644428042, True)))"]]
    bcs = [[InletPressureExtrapolateBC(0, 0), ExtrapolationBC(0, 1, order=0)],
           [IsothermalWallBC(1, 0, [rhoE_wall]), DirichletBC(1, 1, [x_loc] + top)]]
    block.set_block_boundaries(bcs)
    grid = [parse_expr("Eq(DataObject(x0), block.deltas[0]*block.grid_indexes[0])", local_dict=local_dict),
            parse_expr("Eq(DataObject(x1), Lx1*sinh(by*block.deltas[1]*block.grid_indexes[1]/Lx1)/sinh(by))",
                       local_dict=local_dict)]
    fields = ["Eq(GridVariable(w), tanh(DataObject(x1)/5.0))",
              "Eq(GridVariable(u0), w*(1.0 + 0.01*sin(0.05*DataObject(x0))))",
              "Eq(GridVariable(u1), 0.01*w*sin(0.1*DataObject(x0)))",
              "Eq(GridVariable(T), Twall + (1.0 - Twall)*w)",
              "Eq(GridVariable(p), 1.0/(gama*Minf*Minf))",
              "Eq(GridVariable(r), gama*Minf*Minf*p/T)",
              "Eq(DataObject(rho), r)", "Eq(DataObject(rhou0), r*u0)", "Eq(DataObject(rhou1), r*u1)",
              "Eq(DataObject(rhoE), p/(gama-1) + 0.5* r *(u0**2+ u1**2))"]
    local_dict["gama"] = ConstantObject("gama")
    initial = GridBasedInitialisation()
    initial.add_equations(grid + [parse_expr(e, local_dict=local_dict) for e in fields])
    block.set_equations([copy.deepcopy(cr), sim, initial, metriceq])
    block.discretise()
    p = {"gama": "1.4", "Minf": "2.0", "Pr": "0.72", "Re": "950.0", "Twall": "1.67619431",
         "SuthT": "110.4", "RefT": "288.0", "Lx1": "115.0", "by": "5.0",
         "dt": 'osb_env_double("OSB_DT", 0.04)', "niter": 'osb_env_int("OSB_NITER", 1)'}
    for d, (n, dl) in enumerate([(24, "400.0/(block0np0-1)"), (17, "115.0/(block0np1-1)")]):
        p["block0np%d" % d] = 'osb_env_int("OSB_NP%d", %d)' % (d, n)
        p["Delta%dblock0" % d] = dl
    return block, p


def flatten_q(sim):
    from sympy import flatten
    return flatten(sim.time_advance_arrays)


def case_tgv_kgp_tvd():
    """The central KGP TGV of central_split_block followed, after every full RK step, by the
    non-linear characteristic TVD filter (``filters/TVD_filter.py``; Yee-Sandham-Djomehri
    limiter of ``schemes/spatial/shock_capturing.py:619-766``) with its periodic exchange of
    depth 4 -- the ``TVD = True`` branch of
    ``apps/compressible_taylor_green_vortex/compressible_TGV.py:210-222``.  The filter's
    strength kappa_TVD is a run parameter (OSB_KAPPA_TVD)."""
    from opensbli import TVDFilter

    def with_filter(blk):
        wf = TVDFilter(blk, airfoil=False)
        blk.set_equations(wf.equation_classes)
        return wf

    block, params = central_split_block("KGP", "enthalpy", extra=with_filter)
    params["kappa_TVD"] = 'osb_env_double("OSB_KAPPA_TVD", 1.0)'
    return block, params


def case_shock_reflection(formulation=None, flux="LLF", outlet=None):
    """2D inviscid oblique-shock reflection (``apps/inviscid_shock_reflection/inviscid_shock.py``)
    with the app's boundaries -- Dirichlet free-stream inlet, zeroth-order extrapolation outlet,
    symmetry (inviscid wall) bottom, Dirichlet top carrying the post-shock state from x = 40 --
    and its ``weno`` branch with the characteristic LLF WENO5-Z flux (simple average; the app's
    HLLC-LM flux is not on this path) and the standard RK-LS3, or with formulation='SSP' the
    app's own three-stage SSP coefficients (rk_LS.py:102-106)."""
    import copy
    from opensbli import (SimulationBlock, GridBasedInitialisation, GridVariable, DataObject, ConstantObject,
                          parse_expr, SimpleAverage, LFWeno, RungeKuttaLS, DirichletBC, ExtrapolationBC,
                          SymmetryBC)
    ndim = 2
    sim = _euler_equations(ndim, "Weno")
    cr = _constituents(ndim)
    block = SimulationBlock(ndim, block_number=0)
    local_dict = {"block": block, "GridVariable": GridVariable, "DataObject": DataObject}
    for con in ("gama", "Minf"):
        local_dict[con] = ConstantObject(con)
    pe = lambda e: parse_expr(e, local_dict=local_dict)  # noqa: E731
    x0 = pe("Eq(DataObject(x0), block.deltas[0]*block.grid_indexes[0])")
    x1 = pe("Eq(DataObject(x1), block.deltas[1]*block.grid_indexes[1])")
    d_in, u0_in, u1_in = pe("Eq(GridVariable(d), 1.0)"), pe("Eq(GridVariable(u0), 1.0)"), pe("Eq(GridVariable(u1), 0.0)")
    p_in = pe("Eq(GridVariable(p), 1.0/(gama*Minf**2.0))")
    rho, rhou0, rhou1 = pe("Eq(DataObject(rho), d)"), pe("Eq(DataObject(rhou0), d*u0)"), pe("Eq(DataObject(rhou1), d*u1)")
    rhoE = pe("Eq(DataObject(rhoE), p/(gama-1) + 0.5* d *(u0**2+u1**2))")
    initial = GridBasedInitialisation()
    initial.add_equations([x0, x1, d_in, u0_in, u1_in, p_in, rho, rhou0, rhou1, rhoE])
    schemes = {}
    if flux == "LLF":
        LF = LFWeno(order=5, formulation="Z", averaging=SimpleAverage([0, 1]), flux_type="LLF")
    else:
        from opensbli import HLLCWeno
        LF = HLLCWeno(order=5, formulation="Z", averaging=SimpleAverage([0, 1]), flux_type=flux)
    schemes[LF.name] = LF
    rk = RungeKuttaLS(3, formulation=formulation)
    schemes[rk.name] = rk
    block.set_discretisation_schemes(schemes)
    pre, post = 1.0 / (1.4 * 4.0), 1.0 / (1.4 * 4.0) * 1.18646663
    shock_loc = pe("Eq(GridVariable(shock_loc), 40.0)")
    upper = [pe("Eq(GridVariable(x), DataObject(x0))"), shock_loc,
             pe("Eq(GridVariable(d), Piecewise((1.0 ,x<shock_loc),(1.129734572, x>=shock_loc),(1.0,True)))"),
             pe("Eq(GridVariable(u0), Piecewise((1.0 ,x<shock_loc),(0.9667023804242755, x>=shock_loc),(1.0,True)))"),
             pe("Eq(GridVariable(u1), Piecewise((0.0 ,x<shock_loc),(-0.052106102140246795, x>=shock_loc),(1.0,True)))"),
             pe("Eq(GridVariable(p), Piecewise( (%f,x<shock_loc),(%f, x>=shock_loc),(1.0,True)))" % (pre, post)),
             rho, rhou0, rhou1, rhoE]
    if outlet is None:
        right = ExtrapolationBC(0, 1, order=0)
    else:
        from opensbli import PressureOutletBC
        right = PressureOutletBC(0, 1, back_pressure=outlet)
    bcs = [DirichletBC(0, 0, [d_in, u0_in, u1_in, p_in, rho, rhou0, rhou1, rhoE]),
           right, SymmetryBC(1, 0), DirichletBC(1, 1, upper)]
    block.set_block_boundaries(bcs)
    block.set_equations([copy.deepcopy(cr), copy.deepcopy(sim), initial])
    block.discretise()
    p = {"gama": "1.4", "Minf": "2.0", "dt": 'osb_env_double("OSB_DT", 0.1)', "niter": 'osb_env_int("OSB_NITER", 1)',
         "block0np0": 'osb_env_int("OSB_NP0", 457)', "block0np1": 'osb_env_int("OSB_NP1", 255)',
         "Delta0block0": "350.0/(block0np0-1)", "Delta1block0": "115.0/(block0np1-1)"}
    return block, p


def case_kh_weno5z():
    """2D Kelvin-Helmholtz, Euler, characteristic LLF WENO5-Z with Roe average, periodic,
    classic 3-register SBLI RK3 (``apps/kelvin_helmholtz/kelvin_helmholtz.py:20-130``).  The
    HDF5 random-number perturbation of that app is replaced by a deterministic sine mode whose
    amplitude and phase come from the environment (the ensemble draws them from a seeded rng)."""
    import copy
    from opensbli import (SimulationBlock, GridBasedInitialisation, GridVariable, DataObject, parse_expr,
                          RoeAverage, LFWeno, RungeKutta, PeriodicBC)
    ndim = 2
    sim = _euler_equations(ndim, "Weno")
    cr = _constituents(ndim)
    block = SimulationBlock(ndim, block_number=0)
    local_dict = {"block": block, "GridVariable": GridVariable, "DataObject": DataObject}
    eqns = ["Eq(GridVariable(x0), block.deltas[0]*block.grid_indexes[0])",
            "Eq(GridVariable(x1), block.deltas[1]*block.grid_indexes[1])",
            "Eq(GridVariable(d), Piecewise((2.0, Abs(x1 - 0.5) < 0.25), (1.0, True)))",
            "Eq(GridVariable(u0), Piecewise((-0.5, Abs(x1 - 0.5) < 0.25), (0.5, True)))",
            "Eq(GridVariable(u1), 0.01*khamp*sin(4.0*pi*x0 + khphase))",
            "Eq(GridVariable(p), 2.5)",
            "Eq(DataObject(rho), d)", "Eq(DataObject(rhou0), d*u0)", "Eq(DataObject(rhou1), d*u1)",
            "Eq(DataObject(rhoE), p/(gama-1.0) + 0.5*d*(u0**2 + u1**2))"]
    from opensbli.core.opensbliobjects import ConstantObject
    local_dict["khamp"] = ConstantObject("khamp")
    local_dict["khphase"] = ConstantObject("khphase")
    initial = GridBasedInitialisation()
    initial.add_equations([parse_expr(e, local_dict=local_dict) for e in eqns])
    schemes = {}
    LF = LFWeno(5, formulation="Z", averaging=RoeAverage([0, 1]))
    schemes[LF.name] = LF
    rk = RungeKutta(3)
    schemes[rk.name] = rk
    block.set_discretisation_schemes(schemes)
    bcs = []
    for d in range(ndim):
        bcs += [PeriodicBC(d, 0), PeriodicBC(d, 1)]
    block.set_block_boundaries(bcs)
    block.set_equations([copy.deepcopy(cr), copy.deepcopy(sim), initial])
    block.discretise()
    params = {"gama": "1.4", "dt": 'osb_env_double("OSB_DT", 0.0002)', "niter": 'osb_env_int("OSB_NITER", 1)',
              "khamp": 'osb_env_double("OSB_KHAMP", 1.0)', "khphase": 'osb_env_double("OSB_KHPHASE", 0.0)'}
    for d in range(2):
        params["block0np%d" % d] = 'osb_env_int("OSB_NP%d", 32)' % d
        params["Delta%dblock0" % d] = "1.0/block0np%d" % d
    params["block0np2"] = "1"
    return block, params


def case_curv3d_teno5():
    """3D curvilinear Euler on a periodic wavy mesh, characteristic LLF TENO5 (Roe average) with
    4th-order central metrics (MetricsEquation, every direction curvilinear), RK-LS3: the
    single-block form of the 4-block curvilinear configuration's discretisation.  Mesh
    x_i = xi_i Delta_i + 0.05 sin(2 pi eta_j) sin(2 pi eta_k) over the unit box ((i, j, k) cyclic,
    eta = index x Delta), a density / pressure wave rho = 1 + 0.1 sin(2 pi (x0 + x1 + x2)),
    p = 1 / (gama Minf^2) + 0.1 sin(2 pi (x0 - x1)), u = (0.7, -0.3, 0.2)."""
    from sympy import pi, sin, Eq
    from opensbli import (MetricsEquation, EinsteinEquation, SimulationEquations, ConstituentRelations,
                          SimulationBlock, RoeAverage, LFTeno, StoreSome, RungeKuttaLS, GridVariable, DataObject,
                          ConstantObject, parse_expr, GridBasedInitialisation, PeriodicBC)
    ndim = 3
    metriceq = MetricsEquation()
    metriceq.generate_transformations(ndim, "x", [(True, True)] * 3, 2)
    sc1 = "**{'scheme':'Teno'}"
    mass = "Eq(Der(rho,t), - Conservative(detJ * rho*U_j,xi_j,%s)/detJ)" % sc1
    momentum = "Eq(Der(rhou_i,t) , -  Conservative(detJ * (rhou_i*U_j + p*D_j_i), xi_j , %s)/detJ)" % sc1
    energy = "Eq(Der(rhoE,t), - Conservative(detJ * (p+rhoE)*U_j,xi_j, %s)/detJ)" % sc1
    constants_eqns = ["gama", "Minf"]
    einstein = EinsteinEquation()
    einstein.optional_subs_dict = metriceq.metric_subs
    sim = SimulationEquations()
    cr = ConstituentRelations()
    for base in (mass, momentum, energy):
        e = einstein.expand(base, ndim, "xi", [], constants_eqns)
        if base == momentum:
            e = [Eq(x.lhs, x.rhs) for x in e]
        elif base == energy:
            e = Eq(e.lhs, e.rhs)
        sim.add_equations(e)
    for c in ["Eq(u_i, rhou_i/rho)", "Eq(p, (gama-1)*(rhoE-rho*(1/2)*(KD(_i,_j)*u_i*u_j)))",
              "Eq(a, (gama*p/rho)**0.5)", "Eq(U_i, D_i_j*u_j)"]:
        cr.add_equations(einstein.expand(c, ndim, "xi", [], constants_eqns))
    block = SimulationBlock(ndim, block_number=0)
    schemes = {}
    LF = LFTeno(order=5, averaging=RoeAverage([0, 1]), flux_type="LLF")
    schemes[LF.name] = LF
    cent = StoreSome(4, "u0 u1 u2")  # the metric derivatives' central scheme
    schemes[cent.name] = cent
    rk = RungeKuttaLS(3)
    schemes[rk.name] = rk
    block.set_discretisation_schemes(schemes)
    local_dict = {"block": block, "GridVariable": GridVariable, "DataObject": DataObject,
                  "gama": ConstantObject("gama"), "Minf": ConstantObject("Minf")}
    (i, j, k) = block.grid_indexes
    (dx, dy, dz) = block.deltas
    x0 = Eq(DataObject("x0"), i * dx + 0.05 * sin(2.0 * pi * j * dy) * sin(2.0 * pi * k * dz), evaluate=False)
    x1 = Eq(DataObject("x1"), j * dy + 0.05 * sin(2.0 * pi * k * dz) * sin(2.0 * pi * i * dx), evaluate=False)
    x2 = Eq(DataObject("x2"), k * dz + 0.05 * sin(2.0 * pi * i * dx) * sin(2.0 * pi * j * dy), evaluate=False)
    eqs = [parse_expr(e, local_dict=local_dict) for e in [
        "Eq(GridVariable(d), 1+0.1*sin(2*pi*(DataObject(x0)+DataObject(x1)+DataObject(x2))))",
        "Eq(GridVariable(u0), 0.7)", "Eq(GridVariable(u1), -0.3)", "Eq(GridVariable(u2), 0.2)",
        "Eq(GridVariable(p), 1/(gama*Minf**2) + 0.1*sin(2*pi*(DataObject(x0)-DataObject(x1))))",
        "Eq(DataObject(rho), d)", "Eq(DataObject(rhou0), d*u0)", "Eq(DataObject(rhou1), d*u1)",
        "Eq(DataObject(rhou2), d*u2)",
        "Eq(DataObject(rhoE), p/(gama-1) + 0.5* d *(u0**2+u1**2+u2**2))"]]
    initial = GridBasedInitialisation()
    initial.add_equations([x0, x1, x2] + eqs)
    block.set_block_boundaries([[PeriodicBC(d, 0), PeriodicBC(d, 1)] for d in range(ndim)])
    block.set_equations([cr, initial, sim, metriceq])
    block.discretise()
    params = {"gama": "1.4", "Minf": "0.7", "dt": 'osb_env_double("OSB_DT", 0.002)',
              "niter": 'osb_env_int("OSB_NITER", 10)', "TENO_CT": 'osb_env_double("OSB_TENO_CT", 1e-6)'}
    for d, n in enumerate((16, 12, 10)):
        params["block0np%d" % d] = 'osb_env_int("OSB_NP%d", %d)' % (d, n)
        params["Delta%dblock0" % d] = "1.0/(block0np%d)" % d
    return block, params


def case_mb2_flip():
    """Two 2D Euler blocks (characteristic LLF WENO5-Z, simple average, RK-LS3) joined along x by
    two flipped interfaces -- block 0's low-x face to block 1's low-x face and the two high-x
    faces, InterfaceBC(match=(other, 0, side, True)) as the C-mesh wake cut of
    apps/aerofoils/multi_block/2D/airfoil_MB_2D.py:160,170 -- and periodic in y; a different
    smooth state on each block (MultiBlock, TraditionalAlgorithmRKMB)."""
    from opensbli import (MultiBlock, GridBasedInitialisation, GridVariable, DataObject, parse_expr, SimpleAverage,
                          LFWeno, RungeKuttaLS, PeriodicBC, InterfaceBC)
    ndim = 2
    sim = _euler_equations(ndim, "Weno")
    cr = _constituents(ndim)
    mb = MultiBlock(ndim, 2)
    schemes = {}
    LF = LFWeno(order=5, formulation="Z", averaging=SimpleAverage([0, 1]), flux_type="LLF")
    schemes[LF.name] = LF
    rk = RungeKuttaLS(3)
    schemes[rk.name] = rk
    mb.set_discretisation_schemes(schemes)
    bcs = {}
    for b in range(2):
        o = 1 - b
        bcs[b] = [InterfaceBC(direction=0, side=0, halos=[-4, 4], name="b%d_low_x" % b, match=(o, 0, 0, True)),
                  InterfaceBC(direction=0, side=1, halos=[-4, 4], name="b%d_high_x" % b, match=(o, 0, 1, True)),
                  PeriodicBC(1, 0), PeriodicBC(1, 1)]
    mb.set_block_boundaries(bcs)
    inits = {}
    forms = [("1.0 + 0.2*sin(2*pi*(x0 + x1))", "0.4 + 0.1*cos(2*pi*x1)", "-0.2 + 0.1*sin(2*pi*x0)",
              "1.0 + 0.1*cos(2*pi*(x0 - x1))"),
             ("1.1 + 0.15*cos(2*pi*(x0 - 2*x1))", "-0.3 + 0.1*sin(2*pi*(x0 + x1))", "0.25 + 0.1*cos(2*pi*x0)",
              "0.9 + 0.1*sin(2*pi*x1)")]
    for b, blk in enumerate(mb.blocks):
        local_dict = {"block": blk, "GridVariable": GridVariable, "DataObject": DataObject}
        d, u0, u1, p = forms[b]
        eqns = ["Eq(GridVariable(x0), block.deltas[0]*block.grid_indexes[0])",
                "Eq(GridVariable(x1), block.deltas[1]*block.grid_indexes[1])",
                "Eq(GridVariable(d), %s)" % d, "Eq(GridVariable(u0), %s)" % u0, "Eq(GridVariable(u1), %s)" % u1,
                "Eq(GridVariable(p), %s)" % p,
                "Eq(DataObject(rho), d)", "Eq(DataObject(rhou0), d*u0)", "Eq(DataObject(rhou1), d*u1)",
                "Eq(DataObject(rhoE), p/(gama-1.0) + 0.5*d*(u0**2 + u1**2))"]
        init = GridBasedInitialisation()
        init.add_equations([parse_expr(e, local_dict=local_dict) for e in eqns])
        inits[b] = init
    mb.set_equations([cr, sim])
    mb.set_initial_conditions(inits)
    mb.discretise()
    params = {"gama": "1.4", "dt": 'osb_env_double("OSB_DT", 0.0005)', "niter": 'osb_env_int("OSB_NITER", 1)'}
    for b in range(2):
        for d in range(2):
            params["block%dnp%d" % (b, d)] = 'osb_env_int("OSB_NP%d", %d)' % (d, 24 if d == 0 else 20)
            params["Delta%dblock%d" % (d, b)] = "1.0/block%dnp%d" % (b, d)
        params["block%dnp2" % b] = "1"
    return mb, params


def case_curv_weno5z():
    """2D curvilinear wavy-mesh Euler wave, characteristic LLF WENO5-Z (Roe average) with
    4th-order central metrics, periodic, RK-LS3: the reference's verification case
    tests/verification_apps/euler_wave_curvilinear/verify_euler_wave_curvilinear.py (its
    known answer: rho_B0[69,69] = 0.9984292346559068 after 10 steps of dt 5e-4 on 128^2)."""
    from sympy import pi, sin, Eq
    from opensbli import (MetricsEquation, EinsteinEquation, SimulationEquations, ConstituentRelations,
                          SimulationBlock, RoeAverage, LFWeno, StoreSome, RungeKuttaLS, GridVariable, DataObject,
                          ConstantObject, parse_expr, GridBasedInitialisation, PeriodicBC)
    ndim = 2
    metriceq = MetricsEquation()
    metriceq.generate_transformations(ndim, "x", [(True, True), (True, True)], 2)
    sc1 = "**{'scheme':'Weno'}"
    mass = "Eq(Der(rho,t), - Conservative(detJ * rho*U_j,xi_j,%s)/detJ)" % sc1
    momentum = "Eq(Der(rhou_i,t) , -  Conservative(detJ * (rhou_i*U_j + p*D_j_i), xi_j , %s)/detJ)" % sc1
    energy = "Eq(Der(rhoE,t), - Conservative(detJ * (p+rhoE)*U_j,xi_j, %s)/detJ)" % sc1
    constants_eqns = ["gama", "Minf"]
    einstein = EinsteinEquation()
    einstein.optional_subs_dict = metriceq.metric_subs
    sim = SimulationEquations()
    cr = ConstituentRelations()
    for base in (mass, momentum, energy):
        e = einstein.expand(base, ndim, "xi", [], constants_eqns)
        if base == momentum:
            e = [Eq(x.lhs, x.rhs) for x in e]
        elif base == energy:
            e = Eq(e.lhs, e.rhs)
        sim.add_equations(e)
    for c in ["Eq(u_i, rhou_i/rho)", "Eq(p, (gama-1)*(rhoE-rho*(1/2)*(KD(_i,_j)*u_i*u_j)))",
              "Eq(a, (gama*p/rho)**0.5)", "Eq(U_i, D_i_j*u_j)"]:
        cr.add_equations(einstein.expand(c, ndim, "xi", [], constants_eqns))
    block = SimulationBlock(ndim, block_number=0)
    schemes = {}
    LF = LFWeno(5, formulation="Z", averaging=RoeAverage([0, 1]))
    schemes[LF.name] = LF
    cent = StoreSome(4, "u0 u1 T")
    schemes[cent.name] = cent
    rk = RungeKuttaLS(3)
    schemes[rk.name] = rk
    block.set_discretisation_schemes(schemes)
    local_dict = {"block": block, "GridVariable": GridVariable, "DataObject": DataObject,
                  "gama": ConstantObject("gama")}
    (i, j) = block.grid_indexes
    (dx, dy) = block.deltas
    x0 = Eq(DataObject("x0"), i * dx + 0.04 * sin(2.0 * pi * 0.25) * sin(6.0 * pi * j * dy / 2.0), evaluate=False)
    x1 = Eq(DataObject("x1"), j * dy + 0.04 * sin(2.0 * pi * 0.25) * sin(6.0 * pi * i * dx / 2.0), evaluate=False)
    eqs = [parse_expr(e, local_dict=local_dict) for e in [
        "Eq(GridVariable(d), 1+0.2*sin(pi*(DataObject(x0)+DataObject(x1))))", "Eq(GridVariable(u0), 1.0)",
        "Eq(GridVariable(u1), -0.5)", "Eq(GridVariable(p), 1.0)", "Eq(DataObject(rho), d)",
        "Eq(DataObject(rhou0), d*u0)", "Eq(DataObject(rhou1), d*u1)",
        "Eq(DataObject(rhoE), p/(gama-1) + 0.5* d *(u0**2+u1**2))"]]
    initial = GridBasedInitialisation()
    initial.add_equations([x0, x1] + eqs)
    block.set_block_boundaries([[PeriodicBC(d, 0), PeriodicBC(d, 1)] for d in range(ndim)])
    block.set_equations([cr, initial, sim, metriceq])
    block.discretise()
    params = {"gama": "1.4", "dt": 'osb_env_double("OSB_DT", 0.0005)', "niter": 'osb_env_int("OSB_NITER", 10)',
              "block0np0": 'osb_env_int("OSB_NP0", 128)', "block0np1": 'osb_env_int("OSB_NP1", 128)',
              "Delta0block0": "2.0/(block0np0)", "Delta1block0": "2.0/(block0np1)", "block0np2": "1"}
    return block, params


CASES = {
    "sod_weno5js": case_sod_weno5js,
    "sod_extrap": case_sod_extrap,
    "tgv_teno5": lambda: case_tgv_shock("teno5"),
    "tgv_weno5z": lambda: case_tgv_shock("weno5z"),
    "tgv_teno6": lambda: case_tgv_shock("teno6"),
    "tgv_central": case_tgv_central,
    "tgv_kgp": lambda: central_split_block("KGP", "enthalpy"),
    "tgv_kgp_tvd": case_tgv_kgp_tvd,
    "shock_reflection": case_shock_reflection,
    "shock_reflection_ssp": lambda: case_shock_reflection("SSP"),
    "shock_reflection_hllc": lambda: case_shock_reflection("SSP", "HLLC-LM"),
    # the outlet as PressureOutletBC (pressure_outlet.py) with a back pressure of 0.2
    "shock_reflection_pout": lambda: case_shock_reflection(outlet=0.2),
    "kh_weno5z": case_kh_weno5z,
    "curv_weno5z": case_curv_weno5z,
    "curv3d_teno5": case_curv3d_teno5,
    "mb2_flip": case_mb2_flip,
    "channel_iso": case_channel_iso,
    "channel_adi": case_channel_adi,
    "channel_str": lambda: case_channel_iso(stretch=True),
    "channel_tcf": case_channel_tcf,
    "duct_inlet_sub": lambda: case_duct_inlet(0.5),
    "duct_inlet_sup": lambda: case_duct_inlet(2.0),
    "katzer": case_katzer,
}


def build_case(name, reference=None):
    """Build the OpenSBLI block of one case (discretised, no code printed); for tests of the
    drop-in backend.  Returns (block, generator parameter dict)."""
    reference = reference or harness.reference_root()
    if reference is None:
        raise FileNotFoundError("the upstream checkout is not present (set OSB_REFERENCE)")
    if reference not in sys.path:
        sys.path.insert(0, reference)
    apply_compat_patches()
    with open(os.devnull, "w") as dn, contextlib.redirect_stdout(dn):
        return CASES[name]()


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("cases", nargs="*", default=sorted(CASES))
    ap.add_argument("--reference", default=harness.reference_root())
    ap.add_argument("--out", default=os.path.join(HERE, "_ref"))
    args = ap.parse_args(argv)
    if not args.reference or not os.path.isdir(os.path.join(args.reference, "opensbli")):
        print("reference checkout not found at %s; nothing generated" % args.reference)
        return 1
    if len(args.cases) > 1:
        # one interpreter per case: the generator keeps module-level state (the constants to
        # declare, the grid objects), so a case generated after another would inherit its
        # constants; the cases run in parallel
        import concurrent.futures as cf
        cmd = [sys.executable, os.path.abspath(__file__), "--reference", args.reference, "--out", args.out]
        with cf.ThreadPoolExecutor(max_workers=max(1, min(len(args.cases), os.cpu_count() or 1))) as ex:
            rcs = list(ex.map(lambda c: subprocess.call(cmd + [c]), args.cases))
        return max(rcs)
    sys.path.insert(0, args.reference)
    apply_compat_patches()
    for name in args.cases:
        out = os.path.join(args.out, name)
        print("== generating %s -> %s" % (name, out), flush=True)
        with in_dir(out):
            with open(os.devnull, "w") as dn, contextlib.redirect_stdout(dn):
                block, params = CASES[name]()
                _finish(block, {}, params)
    return 0


if __name__ == "__main__":
    sys.exit(main())
