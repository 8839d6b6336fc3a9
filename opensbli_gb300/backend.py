"""Drop-in backend: takes the algorithm object an OpenSBLI problem script builds and runs it on
the GB300 kernels, in place of the OPS C++ printer.

Reference flow (e.g. apps/compressible_taylor_green_vortex/compressible_TGV.py:231-242):

    alg = TraditionalAlgorithmRK(block)
    SimulationDataType.set_datatype(Double)
    OPSC(alg)                                   # writes OPS C++ (opsc.py:407-460)
    substitute_simulation_parameters(names, values)

GB300 flow:

    alg = TraditionalAlgorithmRK(block)
    be = GB300Backend(alg, dict(zip(names, values)))   # precision from SimulationDataType
    be.initialise()                             # the script's GridBasedInitialisation, on the host
    be.run(niter)                               # the generated time loop, on the GPU

The backend walks ``alg.blocks`` and each block's ``discretisation_schemes`` and
``boundary_types`` and maps them onto ``osb_block_desc`` (include/osb_gb300.h).  Anything
outside the supported path (other flux types, other boundary conditions, filters, HLLC ...)
raises ``NotImplementedError``; there is no fallback.
"""
import math

import re

import numpy as np

from . import abi
from .spec import BlockSpec


def _num(expr, params, env=None):
    """Evaluate a simulation-parameter string such as '2*M_PI/block0np0'."""
    if isinstance(expr, (int, float)):
        return float(expr)
    scope = {"M_PI": math.pi, "pi": math.pi, "sqrt": math.sqrt, "ceil": math.ceil}
    if env:
        scope.update(env)
    for k, v in params.items():
        if k not in scope and isinstance(v, (int, float)):
            scope[k] = v
    return float(eval(str(expr), {"__builtins__": {}}, scope))


def resolve_parameters(params):
    """Turn the {name: 'expression'} dict given to substitute_simulation_parameters
    (utilities/helperfunctions.py:150-175) into numbers, resolving cross references."""
    out = {}
    pending = dict(params)
    for _ in range(len(pending) + 1):
        progressed = False
        for k in list(pending):
            try:
                out[k] = _num(pending[k], out)
                del pending[k]
                progressed = True
            except (NameError, TypeError, SyntaxError, ZeroDivisionError):
                continue
        if not pending or not progressed:
            break
    if pending:
        raise ValueError("cannot evaluate simulation parameters: %s" % sorted(pending))
    return out


def _const_value(name, params, default=None):
    if name in params:
        return params[name]
    from opensbli.core.kernel import ConstantsToDeclare
    for c in ConstantsToDeclare.constants:
        if str(c) == name and getattr(c, "value", None) is not None:
            try:
                return float(c.value)
            except (TypeError, ValueError):
                pass
    if default is None:
        raise ValueError("value of constant %s is not known; pass it in the parameters" % name)
    return default


def _flux_of(block):
    """OSB_FLUX_* of the block's shock-capturing scheme: LLF for LFWeno / LFTeno, HLLC-LM for
    HLLCWeno with flux_type 'HLLC-LM' (Cartesian 2D / 3D blocks)."""
    from opensbli.schemes.spatial.weno import HLLCWeno
    for sch in block.discretisation_schemes.values():
        if isinstance(sch, HLLCWeno):
            if getattr(sch, "flux_type", None) != "HLLC-LM":
                raise NotImplementedError("HLLCWeno flux %s is not restated (HLLC-LM is)" % sch.flux_type)
            return abi.FLUX_HLLC_LM
    return abi.FLUX_LLF


def _scheme_of(block):
    """(scheme, averaging, has_central) from block.discretisation_schemes."""
    from opensbli.schemes.spatial.weno import LFWeno, HLLCWeno
    from opensbli.schemes.spatial.teno import LFTeno
    from opensbli.schemes.spatial.scheme import Central
    from opensbli.schemes.spatial.averaging import RoeAverage
    scheme, avg, central = None, abi.AVG_SIMPLE, False
    for sch in block.discretisation_schemes.values():
        if isinstance(sch, (LFWeno, LFTeno, HLLCWeno)):
            if isinstance(sch, (LFWeno, LFTeno)) and getattr(sch, "flux_type", "LLF") != "LLF":
                raise NotImplementedError("only local Lax-Friedrichs splitting is supported (got %s)" % sch.flux_type)
            if getattr(sch, "shock_filter", False):
                raise NotImplementedError("WENO filter steps are not supported")
            owner = getattr(sch.average, "__self__", None)
            avg = abi.AVG_ROE if isinstance(owner, RoeAverage) else abi.AVG_SIMPLE
            if isinstance(sch, LFTeno):
                if sch.order not in (5, 6):
                    raise NotImplementedError("TENO order %d is not supported (TENO5 and TENO6)" % sch.order)
                scheme = abi.SCHEME_TENO5 if sch.order == 5 else abi.SCHEME_TENO6
            else:
                if sch.order != 5:
                    raise NotImplementedError("WENO order %d is not supported (WENO5 only)" % sch.order)
                rv = sch.reconstruction_classes[0]
                is_z = any("Abs" in str(a) for a in rv.alpha_evaluated)
                scheme = abi.SCHEME_WENO5_Z if is_z else abi.SCHEME_WENO5_JS
        elif isinstance(sch, Central):
            if sch.order != 4:
                raise NotImplementedError("central order %d is not supported (4th order only)" % sch.order)
            central = True
    if scheme is None:
        if not central:
            raise NotImplementedError("no supported spatial scheme on block %s" % block.blockname)
        scheme = abi.SCHEME_CENTRAL4
    return scheme, avg, central


def _mu_law(block):
    """(OSB_VISC_SUTHERLAND, 0) for the modified Sutherland mu(T) relation, (OSB_VISC_POWER_LAW,
    e) for mu = T**e (turbulent_channel.py:93), None without a mu relation."""
    from opensbli.equation_types.opensbliequations import ConstituentRelations
    from sympy import flatten, Pow
    for ec in block.list_of_equation_classes:
        if isinstance(ec, ConstituentRelations):
            for eq in flatten(ec.equations):
                if str(eq.lhs).startswith("mu"):
                    rhs = eq.rhs
                    if "1.4042" in str(rhs) and "0.40417" in str(rhs):
                        return abi.VISC_SUTHERLAND, 0.0
                    if isinstance(rhs, Pow) and str(rhs.base).startswith("T") and rhs.exp.is_number:
                        return abi.VISC_POWER_LAW, float(rhs.exp)
                    raise NotImplementedError("viscosity law %s is not supported" % rhs)
    return None


def _viscosity_of(block):
    """OSB_VISC_* from the block's equations: a Sutherland-type or power-law mu(T) constituent
    relation, a constant viscosity (viscous terms without a mu relation), or inviscid."""
    from opensbli.equation_types.opensbliequations import SimulationEquations
    from sympy import flatten
    viscous = False
    for ec in block.list_of_equation_classes:
        if isinstance(ec, SimulationEquations):
            for eq in flatten(ec.equations):
                if "Re" in str(eq.rhs):
                    viscous = True
    law = _mu_law(block)
    if not viscous:
        return abi.VISC_NONE
    return abi.VISC_CONSTANT if law is None else law[0]


def _forcing_of(block, p):
    """(c0, c1, c2) of the channel apps' constant sources (turbulent_channel.py:38-39: "-
    KD(_i,_j)*c_j" in the momentum equations, "- Dot(c_j, u_j)" in the energy equation), None
    when the equations carry no c_j.  Any other use of c_j is refused."""
    from opensbli.equation_types.opensbliequations import SimulationEquations
    from sympy import flatten
    nd = block.ndim
    names = ["c%d" % i for i in range(nd)]
    eqs = [eq for ec in block.list_of_equation_classes if isinstance(ec, SimulationEquations)
           for eq in flatten(ec.equations)]
    syms = {str(x): x for eq in eqs for x in eq.rhs.free_symbols if str(x) in names}
    if not syms:
        return None
    for eq in eqs:
        lhs = str(eq.lhs)
        for i, n in enumerate(names):
            if n not in syms:
                continue
            cf = eq.rhs.expand().coeff(syms[n])
            if "rhoE" in lhs:
                want = r"-u%d(_B\d+)?" % i  # energy (u_i, or its dataset once discretised)
            elif "rhou%d" % i in lhs:
                want = "-1"  # momentum i
            else:
                want = "0"  # mass, the other momentum components
            if not re.fullmatch(want, str(cf)):
                raise NotImplementedError("source term %s * %s in %s is not the channel apps' forcing" % (cf, n, lhs))
    return tuple(float(_const_value(n, p, 0.0)) for n in names) + (0.0,) * (3 - nd)


def _rk_of(block):
    from opensbli.schemes.temporal.rk_LS import RungeKuttaLS
    from opensbli.schemes.temporal.rk_sbli import RungeKutta
    for sch in block.discretisation_schemes.values():
        if isinstance(sch, (RungeKuttaLS, RungeKutta)):
            sch.get_coefficients  # property: fills stage_coeffs / solution_coeffs (rk_LS.py:97-132)
        if isinstance(sch, RungeKuttaLS):
            A = [float(x) for x in sch.stage_coeffs.value]
            B = [float(x) for x in sch.solution_coeffs.value]
            return (abi.RK_LOW_STORAGE, A, B)
        if isinstance(sch, RungeKutta):
            A = [float(x) for x in sch.stage_coeffs.value]
            B = [float(x) for x in sch.solution_coeffs.value]
            return (abi.RK_SBLI3, A, B)
    raise NotImplementedError("no supported time integrator (RungeKuttaLS / RungeKutta)")


def _bcs_of(block, central_only):
    from opensbli.core.boundary_conditions.periodic import PeriodicBC
    from opensbli.core.boundary_conditions.zero_gradient_outlet import ZeroGradientOutletBC
    from opensbli.core.boundary_conditions.extrapolation import ExtrapolationBC
    bc = [[None, None] for _ in range(block.ndim)]
    depth = [[4, 4] for _ in range(block.ndim)]
    flips = [[None, None] for _ in range(block.ndim)]
    for d, pair in enumerate(block.boundary_types):
        for side, b in enumerate(pair):
            if isinstance(b, PeriodicBC):
                bc[d][side] = abi.BC_PERIODIC
                if b.halos is not None:
                    depth[d][side] = abs(b.halos[side])
                else:
                    hv = b.get_halo_values(block)
                    depth[d][side] = abs(hv[d][side])
            elif isinstance(b, ZeroGradientOutletBC):
                bc[d][side] = abi.BC_ZERO_GRAD
                hv = b.get_halo_values(block)
                depth[d][side] = abs(hv[d][side])
            elif isinstance(b, ExtrapolationBC):
                if b.order not in (0, 1):
                    raise NotImplementedError("extrapolation of order %s is not supported" % b.order)
                bc[d][side] = abi.BC_EXTRAP0 if b.order == 0 else abi.BC_EXTRAP1
                hv = b.get_halo_values(block)
                depth[d][side] = abs(hv[d][side])
            elif type(b).__name__ == "SymmetryBC":
                bc[d][side] = abi.BC_SYMMETRY
                hv = b.get_halo_values(block)
                depth[d][side] = abs(hv[d][side])
            elif type(b).__name__ == "PressureOutletBC":
                bc[d][side] = abi.BC_PRESSURE_OUTLET
                hv = b.get_halo_values(block)
                depth[d][side] = abs(hv[d][side])
            elif type(b).__name__ == "IsothermalWallBC":
                # isothermal_wall.py:62-131; its wall energy equation is read by wall_temperature
                bc[d][side] = abi.BC_ISOTHERMAL_WALL
                hv = b.get_halo_values(block)
                depth[d][side] = abs(hv[d][side])
            elif type(b).__name__ == "AdiabaticWallBC":
                bc[d][side] = abi.BC_ADIABATIC_WALL  # adiabatic_wall.py:28-69
                hv = b.get_halo_values(block)
                depth[d][side] = abs(hv[d][side])
            elif type(b).__name__ == "SharedInterfaceBC":
                raise NotImplementedError("SharedInterfaceBC (interfaces sharing their boundary points) is not "
                                          "implemented; InterfaceBC is")
            elif type(b).__name__ == "InterfaceBC":
                # multi_block.py:48-107: the neighbour's layers next to its face fill this face's
                # halos, in reverse order along the normal when the match flag is set
                # (opsc.py:1043-1045); depth = the neighbour's scheme halo on that side
                match = tuple(b.match)
                if len(match) < 3 or match[1] != d:
                    raise NotImplementedError("interface of direction %d matched to direction %s of block %s: only "
                                              "faces normal to the same direction are implemented" % (
                                                  d, match[1] if len(match) > 1 else None, match[0]))
                bc[d][side] = abi.BC_INTERFACE
                flips[d][side] = (int(match[0]), int(match[1]), int(match[2]),
                                  1 if len(match) > 3 and match[3] else 0)
                hv = b.get_halo_values(block)
                depth[d][side] = abs(hv[d][side])
            elif type(b).__name__ == "DirichletBC":
                # the generated kernel covers the plane and the scheme's halo on that side
                # (dirichlet.py:35-40: block.boundary_halos)
                bc[d][side] = abi.BC_DIRICHLET
                depth[d][side] = max(abs(h.get_halos(side)) for h in block.boundary_halos[d][side])
            else:
                raise NotImplementedError("boundary condition %s is not supported" % type(b).__name__)
    return bc, depth, flips


def _rhs_names(eqn):
    """Names of the data objects on the right-hand side of one expanded equation."""
    return {str(a) for a in eqn.rhs.atoms() if type(a).__name__ in ("DataObject", "Symbol")}


def _split_form_of(block):
    """Convective split form of a central-scheme block (physical_models/split_forms.py), read
    from its expanded simulation equations.  Over the reference's forms (Divergence, Blaisdell,
    Feiereisen, Jameson, Kok, KGP, KEEP, each with either energy formulation) the symbol sets
    of the continuity and energy right-hand sides single out the two implemented ones:
      Feiereisen: continuity holds only rhou_j; energy holds rhoE, rho, rhou_j, p and neither H
                  nor e;
      KGP (enthalpy formulation): continuity holds rho, u_j, rhou_j; energy holds H and rho and
                  none of p, rhoE, e.
    Any other form raises NotImplementedError."""
    from opensbli import SimulationEquations
    from sympy import flatten
    eqs = []
    for ec in block.list_of_equation_classes:
        if isinstance(ec, SimulationEquations):
            eqs += flatten(ec.equations)
    by_lhs = {}
    for e in eqs:
        name = str(getattr(e.lhs, "args", [e.lhs])[0]) if getattr(e.lhs, "args", None) else str(e.lhs)
        by_lhs[name.split("_B")[0]] = e
    mass, energy = by_lhs.get("rho"), by_lhs.get("rhoE")
    if mass is None or energy is None:
        raise NotImplementedError("central scheme: continuity / energy equations not found")
    m, en = _rhs_names(mass), _rhs_names(energy)
    nd = block.ndim
    rhou = {"rhou%d" % i for i in range(nd)}
    u = {"u%d" % i for i in range(nd)}
    if m <= rhou and {"rhoE", "rho", "p"} <= en and rhou <= en and not ({"H", "e"} & en):
        return abi.SPLIT_FEIEREISEN
    if ({"rho"} | u | rhou) <= m and {"H", "rho"} <= en and not ({"p", "rhoE", "e"} & en):
        return abi.SPLIT_KGP
    raise NotImplementedError("central convective split form not supported (Feiereisen and KGP with the enthalpy "
                              "energy formulation are); continuity uses %s, energy %s" % (sorted(m), sorted(en)))


# Kernel names the non-linear filters give their equation classes (filters/TVD_filter.py:66,
# 91, 142; filters/WENO_filter.py:301-351, 468, 503, 555).
_TVD_KERNELS = ("TVD reconstruction direction", "Non-linear TVD Filter application")
_WENO_FILTER_KERNELS = ("WENO reconstruction direction", "Non-linear filter application")


def _kernel_names(ec):
    return [str(getattr(k, "computation_name", "")) for k in getattr(ec, "Kernels", [])]


def _filter_of(block, p):
    """(OSB_FILTER_*, kappa_TVD) of the non-linear filter whose equation classes the block
    carries.  The TVD filter of filters/TVD_filter.py without its hybrid sensor
    (optimize=False, the TGV app's TVD branch) maps onto OSB_FILTER_TVD with the run's
    kappa_TVD; its sensor variant and the WENO filter fail loudly here (the WENO filter's
    Central4-WENO5 form is reached through BlockSpec, problems.tgv_filtered)."""
    names = [n for ec in block.list_of_equation_classes for n in _kernel_names(ec)]
    tvd = any(any(t in n for t in _TVD_KERNELS) for n in names)
    weno = any(any(t in n for t in _WENO_FILTER_KERNELS) for n in names)
    if weno:
        raise NotImplementedError("the WENO filter of filters/WENO_filter.py is not mapped by the backend; "
                                  "its Central4-WENO5 form is reached through BlockSpec (problems.tgv_filtered)")
    if not tvd:
        return abi.FILTER_NONE, 1.0
    if any("Shock sensor" in n for n in names):
        raise NotImplementedError("the TVD filter with its Ducros sensor (TVDFilter(optimize=True)) is not "
                                  "implemented; the unsensored filter is")
    for name, fixed in (("delta_TVD", 0.5), ("eps_TVD", 1.0e-8)):
        if name in p and float(p[name]) != fixed:
            raise NotImplementedError("%s = %s: the TVD filter is implemented for the generator's %s" % (
                name, p[name], fixed))
    return abi.FILTER_TVD, float(_const_value("kappa_TVD", p))


def _check_equation_classes(block):
    """Fail loudly on equation classes the GB300 path does not run (explicit filters and
    others), instead of ignoring them.  The non-linear filters' own classes are recognised by
    _filter_of."""
    from opensbli import SimulationEquations, ConstituentRelations, GridBasedInitialisation
    allowed = (SimulationEquations, ConstituentRelations, GridBasedInitialisation)
    for ec in block.list_of_equation_classes:
        if isinstance(ec, allowed):
            continue
        name = type(ec).__name__
        if name == "MetricsEquation":
            continue  # evaluated by metrics_of: the block becomes curvilinear, its metrics computed on the GPU
        if name == "UserDefinedEquations":
            continue  # a non-linear filter's kernels (_filter_of) or post-processing reductions
        raise NotImplementedError("equation class %s is not supported by the GB300 backend%s" % (
            name, "; the non-linear WENO filter is reached through BlockSpec (problems.tgv_filtered)"
            if "filter" in name.lower() or "Filter" in name else ""))


def metrics_of(block):
    """Coordinate names (x0, x1[, x2]) of a block that carries a MetricsEquation
    (equation_types/metric.py:24-451), None for a Cartesian block.

    The supported form is the one the curvilinear apps use: every direction curvilinear
    (generate_transformations(ndim, 'x', [(True, True)] * ndim, order), so the ten arrays are
    D = adj(J) / det J and det J of J_ij = d x_i / d xi_j, metric.py:183-197), the non-conservative
    metrics, on a block whose faces are all periodic (the metric kernel runs over the interior and
    the arrays are exchanged like the state).  Stretched-only or Cartesian directions, the
    conservative metrics, and non-periodic curvilinear blocks (whose metric derivatives take the
    one-sided boundary closures of Carpenter_scheme.py) raise NotImplementedError."""
    mets = [ec for ec in block.list_of_equation_classes if type(ec).__name__ == "MetricsEquation"]
    if not mets:
        return None
    me = mets[0]
    if ystretch_of(block) is not None:
        return None  # the stretched wall-normal grid: a Cartesian block with D11 / SD111 rows
    if not all(getattr(me, "curvilinear_metric", [])) or len(me.curvilinear_metric) != block.ndim:
        raise NotImplementedError("MetricsEquation with stretched-only or Cartesian directions (%s) is not supported; "
                                  "every direction must be curvilinear" % (getattr(me, "curvilinear_metric", None),))
    if getattr(me, "conservative_metrics", False):
        raise NotImplementedError("conservative metrics are not supported")
    from opensbli.core.boundary_conditions.periodic import PeriodicBC
    for d, pair in enumerate(block.boundary_types):
        for side, b in enumerate(pair):
            if not isinstance(b, PeriodicBC):
                raise NotImplementedError(
                    "curvilinear block with a %s face (direction %d side %d): the metric derivatives at non-periodic "
                    "boundaries need the one-sided Carpenter closures, which are not implemented" % (
                        type(b).__name__, d, side))
    return [str(c) for c in me.cartesian_coordinates]


def ystretch_of(block):
    """Coordinate name of the wall-normal direction (x1) of a 3D block whose MetricsEquation
    stretches direction 1 only (generate_transformations(3, 'x', [(False, False), (True, False),
    (False, False)], 2), metric.py:43-64, applied to the equations: the form of
    apps/channel_flow/compressible_TCF_TENO/turbulent_channel.py:225-228), None otherwise."""
    mets = [ec for ec in block.list_of_equation_classes if type(ec).__name__ == "MetricsEquation"]
    if not mets or block.ndim != 3:
        return None
    me = mets[0]
    if any(getattr(me, "curvilinear_metric", [True])) or list(getattr(me, "stretching_metric", [])) != [False, True,
                                                                                                         False]:
        return None
    return str(me.cartesian_coordinates[1])


def _ystretch_rows(block, spec, params, name):
    """(D11, SD111) of the wall-normal grid line the block's initialisation defines
    (abi.ystretch_metrics, the generated metric kernels); the line must not vary in x or z."""
    x1 = coordinates(block, spec, params, [name])[0]
    sl = spec.interior()
    h = spec.halo
    line = np.ascontiguousarray(x1[h, h:h + spec.size[1], h])
    if not np.array_equal(x1[sl], np.broadcast_to(line[None, :, None], x1[sl].shape)):
        raise NotImplementedError("a stretched y grid whose %s varies in x or z is not supported" % name)
    return abi.ystretch_metrics(line, spec.delta[1], spec.bc[1][0] in (abi.BC_ISOTHERMAL_WALL, abi.BC_ADIABATIC_WALL),
                                spec.bc[1][1] in (abi.BC_ISOTHERMAL_WALL, abi.BC_ADIABATIC_WALL))


def _teno_eps(p):
    """The TENO epsilon of the generated code: LFTeno gives its 'eps' constant the value 1e-40
    (teno.py:368-371), which the code printer writes as a literal; parameter substitution only
    fills constants declared without a value ('=Input', helperfunctions.py:150-175), so a script's
    own 'eps' parameter (the TENO channel app passes 1e-15) does not reach the solver."""
    from opensbli.core.kernel import ConstantsToDeclare
    for c in ConstantsToDeclare.constants:
        if str(c) == "eps" and getattr(c, "value", None) is not None:
            return float(c.value)
    return _const_value("eps", p, 1e-40)


def block_spec(block, params):
    """BlockSpec of one OpenSBLI SimulationBlock."""
    p = resolve_parameters(params)
    b = block.blocknumber
    nd = block.ndim
    size = tuple(int(_const_value("block%dnp%d" % (b, d), p)) for d in range(nd))
    delta = tuple(float(_const_value("Delta%dblock%d" % (d, b), p)) for d in range(nd))
    scheme, avg, central = _scheme_of(block)
    _check_equation_classes(block)
    coords = metrics_of(block)
    visc = _viscosity_of(block)
    if coords is not None and (visc != abi.VISC_NONE or scheme == abi.SCHEME_CENTRAL4):
        raise NotImplementedError("curvilinear blocks take the characteristic Euler flux only (the metric-"
                                  "transformed central and viscous terms are not implemented)")
    bc, depth, iface = _bcs_of(block, scheme == abi.SCHEME_CENTRAL4)
    split = _split_form_of(block) if scheme == abi.SCHEME_CENTRAL4 else abi.SPLIT_FEIEREISEN
    filt, kappa = _filter_of(block, p)
    spec = BlockSpec(ndim=nd, size=size, scheme=scheme, averaging=avg, viscous=visc, bc=bc, bc_depth=depth,
                     iface=iface if any(f is not None for pair in iface for f in pair) else None,
                     split_form=split, filter=filt, tvd_kappa=kappa, flux_type=_flux_of(block),
                     gama=_const_value("gama", p), Minf=_const_value("Minf", p, 1.0), Re=_const_value("Re", p, 1.0),
                     Pr=_const_value("Pr", p, 0.71), mu_const=1.0, eps=_teno_eps(p),
                     teno_ct=_const_value("TENO_CT", p, 1e-6),
                     shock_filter_control=_const_value("shock_filter_control", p, 1.0), delta=delta,
                     curvilinear=coords is not None)
    if any(k == abi.BC_DIRICHLET for pair in bc for k in pair):
        spec.dirichlet = dirichlet_faces(block, spec, params)
    outlets = {(d, side): float(b.back_pressure) for d, pair in enumerate(block.boundary_types)
               for side, b in enumerate(pair) if bc[d][side] == abi.BC_PRESSURE_OUTLET}
    if outlets:
        spec.back_pressure = outlets
    walls = {(d, side): wall_temperature(b, spec, params) for d, pair in enumerate(block.boundary_types)
             for side, b in enumerate(pair) if bc[d][side] == abi.BC_ISOTHERMAL_WALL}
    if walls:
        spec.wall_temperature = walls
    law = _mu_law(block)
    if visc == abi.VISC_POWER_LAW:
        spec.visc_power = law[1]
    forcing = _forcing_of(block, p)
    if forcing is not None and any(forcing):
        spec.forcing = forcing
    ycoord = ystretch_of(block)
    if ycoord is not None:
        wall = (abi.BC_ISOTHERMAL_WALL, abi.BC_ADIABATIC_WALL)
        if visc == abi.VISC_NONE or bc[1][0] not in wall or bc[1][1] not in wall:
            raise NotImplementedError("a stretched y grid is implemented for viscous blocks with walls on both y faces")
        spec.ystretch = _ystretch_rows(block, spec, params, ycoord)
    return spec


def wall_temperature(bc, spec, params):
    """Twall of an IsothermalWallBC whose equation sets the wall energy to
    rhoE = Twall rho / (gama Minf^2 (gama - 1)) (the wall of the channel and SBLI apps, e.g.
    apps/channel_flow/compressible_TCF_Central/turbulent_channel.py:118-131): the equation is
    evaluated at two wall densities and must be that linear law; other wall equations raise."""
    import sympy
    from opensbli.core.opensbliobjects import DataSet, ConstantObject
    eqs = list(bc.equations)
    if len(eqs) != 1 or not str(getattr(eqs[0].lhs, "base", eqs[0].lhs)).startswith("rhoE"):
        raise NotImplementedError("IsothermalWallBC: only the wall-energy equation rhoE = Twall*rho/(gama*Minf**2*"
                                  "(gama-1)) is supported")
    rhs = eqs[0].rhs
    p = resolve_parameters(params)
    rho = [a for a in rhs.atoms(DataSet) if str(a.base).split("_")[0] == "rho"]
    other = [a for a in rhs.atoms(DataSet) if a not in rho]
    if len(rho) != 1 or other:
        raise NotImplementedError("IsothermalWallBC: the wall energy must depend on the wall density alone")

    def at(r):  # the wall energy at wall density r (the data set first: its indices hold constants)
        e = rhs.subs(rho[0], r)
        return float(e.subs({a: _const_value(str(a), p) for a in e.atoms(ConstantObject)}))
    scale = spec.gama * spec.Minf ** 2 * (spec.gama - 1.0)
    t1 = at(1.0) * scale
    t2 = at(2.0) * scale / 2.0
    if not (t1 > 0.0) or abs(t1 - t2) > 1e-12 * abs(t1) or not sympy.Float(t1).is_finite:
        raise NotImplementedError("IsothermalWallBC: the wall energy is not Twall*rho/(gama*Minf**2*(gama-1))")
    # the value of the equation's temperature constant itself (t1 carries the rounding of the
    # evaluation above)
    for a in rhs.atoms(ConstantObject):
        if str(a) in ("gama", "Minf"):
            continue
        v = _const_value(str(a), p, default=float("nan"))
        if abs(v - t1) <= 1e-12 * abs(t1):
            return float(v)
    return t1


def initial_state(block, spec, params):
    """Evaluate the block's GridBasedInitialisation equations on the host over every allocated
    point (the generated initialisation kernel's range -halo..N+halo), returning the
    conserved variables in OPS layout."""
    values = _initial_values(block, spec, params)
    order = ["rho"] + ["rhou%d" % d for d in range(spec.ndim)] + ["rhoE"]
    return [np.ascontiguousarray(values[n]) for n in order]


def dirichlet_faces(block, spec, params):
    """Values of every DirichletBC face of the block on its boundary plane and halo layers, in
    the layout osb_block_desc.dirichlet takes ([v][layer][t]): the BC's equations evaluated over
    the allocation with the data objects the initialisation defines (the grid coordinates x0,
    x1, ...), as the generated boundary kernel reads them."""
    faces = {}
    init = None
    h = spec.halo
    for d, pair in enumerate(block.boundary_types):
        for side, b in enumerate(pair):
            if spec.bc[d][side] != abi.BC_DIRICHLET:
                continue
            if init is None:
                init = _initial_values(block, spec, params)
            vals = _initial_values(block, spec, params, equations=b.equations, values=dict(init))
            order = ["rho"] + ["rhou%d" % e for e in range(spec.ndim)] + ["rhoE"]
            depth = spec.bc_depth[d][side]
            ax = spec.ndim - 1 - d
            n = spec.size[d]
            first = h - depth if side == 0 else h + n - 1
            out = []
            for name in order:
                a = np.moveaxis(np.asarray(vals[name]), ax, 0)[first:first + depth + 1]
                # [layer][other axes, slowest first] -> [layer][t] with the lower direction fastest
                out.append(a.reshape(depth + 1, -1))
            faces[(d, side)] = np.ascontiguousarray(np.stack(out))
    return faces


def _initial_values(block, spec, params, equations=None, values=None):
    """Evaluate equations (default: the block's GridBasedInitialisation) over every allocated
    point with numpy; returns {name: array} of everything they define."""
    import sympy
    from sympy import flatten
    from opensbli.initialisation.gridbasedinit import GridBasedInitialisation
    p = resolve_parameters(params)
    if equations is None:
        inits = [ec for ec in block.list_of_equation_classes if isinstance(ec, GridBasedInitialisation)]
        if not inits:
            raise NotImplementedError("block has no GridBasedInitialisation")
        equations = flatten([e.equations for e in inits])
    env = {}
    idx = [spec.grid_index(d).astype(np.float64) for d in range(spec.ndim)]
    for d in range(spec.ndim):
        env[str(block.grid_indexes[d])] = idx[d]
        env[str(block.deltas[d])] = spec.delta[d]
    for k, v in p.items():
        env.setdefault(k, v)
    mods = [{"Abs": np.abs, "Piecewise": _np_piecewise}, "numpy"]
    values = {} if values is None else values
    for eq in flatten(equations):
        lhs, rhs = eq.lhs, eq.rhs
        indexed = sorted(rhs.atoms(sympy.Indexed), key=str)
        dummies = {ix: sympy.Symbol("_ix%d" % i) for i, ix in enumerate(indexed)}
        body = rhs.subs(dummies)
        back = {v: k for k, v in dummies.items()}
        syms = sorted(body.free_symbols, key=str)
        args = []
        for sym in syms:
            n = str(back.get(sym, sym))
            key = n.split("[")[0]
            base = key[:-3] if key.endswith("_B%d" % block.blocknumber) else key
            for cand in (n, key, base):
                if cand in values:
                    args.append(values[cand])
                    break
                if cand in env:
                    args.append(env[cand])
                    break
            else:
                raise ValueError("initial condition uses unknown symbol %s" % n)
        f = sympy.lambdify(syms, body, modules=mods)
        val = f(*args)
        name = str(lhs).split("[")[0]
        name = name[:-3] if name.endswith("_B%d" % block.blocknumber) else name
        values[name] = np.broadcast_to(np.asarray(val, dtype=np.float64), spec.shape)
    return values


def _np_piecewise(*args):
    out = None
    for expr, cond in reversed(args):
        if out is None:
            out = np.asarray(expr, dtype=np.float64) * np.ones_like(np.asarray(cond, dtype=np.float64))
        else:
            out = np.where(cond, expr, out)
    return out


PRECISION_STRATEGIES = ("q_vector", "wk_arrays", "residuals", "RK_arrays", "custom")


def precision_of(mixed_precision_config=None):
    """Precision mode implied by the reference's own precision knobs.

    The reference stores every dataset in one global type (``SimulationDataType.set_datatype``,
    core/datatypes.py:3-17: Double or FloatC; Half exists as a type) and can lower the storage
    of groups of arrays (``OPSC(..., mixed_precision_config={strategy: (arrays, type)})``,
    code_generation/opsc.py:462-534, strategies q_vector, wk_arrays, residuals, RK_arrays,
    custom).  Here the state, the RK registers and the reductions are always FP64 and what can
    be lowered is the arithmetic of the residual, so:

    * Double everywhere (or nothing set) -> "fp64";
    * FloatC globally or for any strategy -> "fp32" (FP32 residual; no array ends up with
      less precision than the script asked for);
    * Half anywhere -> NotImplementedError;
    * an unknown strategy -> ValueError, as opsc.py:523 raises (the keyword itself is
      OPSC.__init__, opsc.py:408).
    """
    from opensbli.core.datatypes import DataType, FloatC, Half, SimulationDataType
    types = []
    glob = SimulationDataType.__dict__.get("dtype")
    if isinstance(glob, type) and issubclass(glob, DataType):
        types.append(glob)
    for strategy, inputs in (mixed_precision_config or {}).items():
        if strategy not in PRECISION_STRATEGIES:
            raise ValueError("Unknown mixed precision preset: {}. Please choose from: {}."
                             .format(strategy, ", ".join(PRECISION_STRATEGIES)))
        types.append(inputs[1])
    for t in types:
        if isinstance(t, type) and issubclass(t, Half):
            raise NotImplementedError("half-precision storage is not supported (FP32 residual is the lowest)")
    return "fp32" if any(isinstance(t, type) and issubclass(t, FloatC) for t in types) else "fp64"


def coordinates(block, spec, params, names):
    """Grid coordinates (the DataObjects the block's GridBasedInitialisation defines under the
    MetricsEquation's coordinate names) at every allocated point, OPS layout."""
    values = _initial_values(block, spec, params)
    missing = [n for n in names if n not in values]
    if missing:
        raise NotImplementedError("curvilinear block: the initialisation does not define the coordinates %s" % missing)
    return [np.ascontiguousarray(values[n], dtype=np.float64) for n in names]


class BackendPlan:
    """What GB300Backend derives from an OpenSBLI algorithm: per block its BlockSpec, its initial
    state (the GridBasedInitialisation evaluated over the allocation) and, for a curvilinear
    block, its grid coordinates; the time integrator (kind, A, B); dt, niter and the precision.
    It holds plain arrays only, so it can be written to a file (save) and run where the
    OpenSBLI generator is not installed (GB300Backend.from_plan)."""

    def __init__(self, specs, states, coords, rk, dt=None, niter=None, precision="fp64"):
        self.specs = list(specs)
        self.states = [None if q is None else [np.ascontiguousarray(a, dtype=np.float64) for a in q] for q in states]
        self.coords = [None if x is None else [np.ascontiguousarray(a, dtype=np.float64) for a in x] for x in coords]
        kind, A, B = rk
        self.rk = (int(kind), tuple(float(x) for x in A), tuple(float(x) for x in B))
        self.dt = None if dt is None else float(dt)
        self.niter = None if niter is None else int(niter)
        self.precision = precision

    def save(self, path):
        """One .npz: a JSON record of the specs and scalars plus the arrays."""
        import json
        arrays = {}
        recs = []
        for ib, spec in enumerate(self.specs):
            rec, arr = spec.to_record()
            recs.append(rec)
            for k, a in arr.items():
                arrays["b%d_%s" % (ib, k)] = a
            for v, a in enumerate(self.states[ib] or []):
                arrays["b%d_q%d" % (ib, v)] = a
            for d, a in enumerate(self.coords[ib] or []):
                arrays["b%d_x%d" % (ib, d)] = a
        meta = {"specs": recs, "rk": [self.rk[0], list(self.rk[1]), list(self.rk[2])], "dt": self.dt,
                "niter": self.niter, "precision": self.precision,
                "ncoords": [0 if x is None else len(x) for x in self.coords]}
        np.savez_compressed(path, meta=np.array(json.dumps(meta)), **arrays)

    @classmethod
    def load(cls, path):
        import json
        with np.load(path) as f:
            meta = json.loads(str(f["meta"]))
            specs, states, coords = [], [], []
            for ib, rec in enumerate(meta["specs"]):
                pre = "b%d_" % ib
                arr = {k[len(pre):]: f[k] for k in f.files
                       if k.startswith(pre + "dirichlet_") or k.startswith(pre + "ystretch_")}
                spec = BlockSpec.from_record(rec, arr)
                specs.append(spec)
                states.append([f[pre + "q%d" % v] for v in range(spec.nvars)])
                nc = meta["ncoords"][ib]
                coords.append([f[pre + "x%d" % d] for d in range(nc)] if nc else None)
        rk = (meta["rk"][0], meta["rk"][1], meta["rk"][2])
        return cls(specs, states, coords, rk, meta["dt"], meta["niter"], meta["precision"])


class GB300Backend:
    """Stands in for OPSC(alg): owns the GPU state of every block of ``alg`` and runs its
    time loop on the GB300 kernels.  ``precision`` is "fp64" or "fp32" (FP32 residual, FP64
    state); left as None it follows the script's SimulationDataType and the optional
    ``mixed_precision_config`` of OPSC (see precision_of).

    A curvilinear block (a MetricsEquation, see metrics_of) gets its ten metric arrays computed
    on the GPU from the grid coordinates its initialisation defines (osb_metrics, the generated
    metric kernel's central differences, halos from the periodic images) and passed with the
    block; it is never run as a Cartesian block.  ``plan()`` returns everything the backend
    derived from the algorithm as a BackendPlan; ``GB300Backend.from_plan`` runs such a plan
    without the OpenSBLI generator (initialise and run are the same code)."""

    def __init__(self, alg, parameters, precision=None, device=0, graphs=True, mixed_precision_config=None,
                 blocks=None):
        """alg: what the script would hand to OPSC -- TraditionalAlgorithmRK(block), or for a
        MultiBlock problem the MultiBlock itself or TraditionalAlgorithmRKMB(multi_block) with
        blocks=multi_block (that algorithm object keeps no reference to its blocks)."""
        if precision is None:
            precision = precision_of(mixed_precision_config)
        if precision not in ("fp64", "fp32"):
            raise ValueError("precision must be 'fp64' or 'fp32', not %r" % (precision,))
        self.alg = alg
        self.params = dict(parameters)
        self.numbers = resolve_parameters(self.params)
        if blocks is not None:
            self.blocks = list(getattr(blocks, "blocks", blocks))
        elif hasattr(alg, "blocks"):
            self.blocks = list(alg.blocks)
        else:
            raise ValueError("a multi-block algorithm keeps no reference to its blocks: pass blocks=multi_block")
        self.specs = [block_spec(b, self.params) for b in self.blocks]
        for s in self.specs[1:]:
            if not s.same_discretisation(self.specs[0]):
                raise NotImplementedError("blocks with different discretisations")
        self.coord_names = [metrics_of(b) for b in self.blocks]
        self.rk = _rk_of(self.blocks[0])
        self.precision = precision
        self.device = device
        self.graphs = graphs
        self.dt = float(self.numbers["dt"]) if "dt" in self.numbers else None
        self.niter = int(self.numbers["niter"]) if "niter" in self.numbers else None
        self.solver = None
        self.metrics = None
        self.iteration = 0
        self.simulation_time = 0.0
        self._plan = None

    @classmethod
    def from_plan(cls, plan, precision=None, device=0, graphs=True):
        """A backend that runs a BackendPlan (plan.precision unless precision is given)."""
        be = cls.__new__(cls)
        be.alg = None
        be.params = {}
        be.numbers = {}
        be.blocks = []
        be.specs = list(plan.specs)
        be.coord_names = [None if x is None else ["x%d" % d for d in range(len(x))] for x in plan.coords]
        be.rk = plan.rk
        be.precision = precision or plan.precision
        if be.precision not in ("fp64", "fp32"):
            raise ValueError("precision must be 'fp64' or 'fp32', not %r" % (be.precision,))
        be.device = device
        be.graphs = graphs
        be.dt = plan.dt
        be.niter = plan.niter
        be.solver = None
        be.metrics = None
        be.iteration = 0
        be.simulation_time = 0.0
        be._plan = plan
        return be

    def plan(self):
        """The BackendPlan of this algorithm: specs, initial states, coordinates, RK, dt, niter."""
        if self._plan is None:
            states = [initial_state(b, s, self.params) for b, s in zip(self.blocks, self.specs)]
            coords = [None if names is None else coordinates(b, s, self.params, names)
                      for b, s, names in zip(self.blocks, self.specs, self.coord_names)]
            self._plan = BackendPlan(self.specs, states, coords, self.rk, self.dt, self.niter, self.precision)
        return self._plan

    def initialise(self, states=None, restart=None):
        """Upload the initial state (default: the scripts' GridBasedInitialisation evaluated on the
        host), compute the metric arrays of curvilinear blocks on the GPU, and apply the boundary
        conditions once, as the generated code does before its time loop.  restart: a file
        written by save(); its state, RK register, iteration and simulation time replace the
        initialisation (the generated code's restart == 1 branch, opsc.py:962-977)."""
        from .solver import Solver, device_metrics
        plan = self.plan()
        if states is None:
            states = plan.states
        self.metrics = []
        for spec, x in zip(self.specs, plan.coords):
            if spec.curvilinear != (x is not None):
                raise abi.OSBError("block curvilinear flag and coordinates disagree")
            self.metrics.append(None if x is None else
                                device_metrics(spec, x, fill=abi.METRIC_PERIODIC, device=self.device))
        items = [(s, q) if m is None else (s, q, m) for s, q, m in zip(self.specs, states, self.metrics)]
        self.solver = Solver(items, precision=self.precision, rk=self.rk, device=self.device, graphs=self.graphs)
        if restart is not None:
            self.iteration, self.simulation_time = self.solver.load_restart(restart)
        self.solver.apply_bc()
        return self

    def save(self, path):
        """Write a restart file (state, RK register, iteration, simulation time of every block)."""
        self.solver.save_restart(path, self.iteration, self.simulation_time)

    def run(self, niter=None, dt=None):
        niter = self.niter if niter is None else niter
        dt = self.dt if dt is None else dt
        if niter is None or dt is None:
            raise ValueError("niter and dt must be given (as parameters or arguments)")
        self.solver.step(dt, niter)
        self.iteration += niter
        self.simulation_time += niter * dt
        self.solver.sync()
        return self

    def state(self, ib=0):
        return self.solver.state(ib)

    def reduce(self, what):
        return self.solver.reduce(what)

    def close(self):
        if self.solver is not None:
            self.solver.close()
            self.solver = None
