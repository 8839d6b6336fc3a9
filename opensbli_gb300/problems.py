"""Synthetic workloads: block specifications and initial conditions of the parity and
benchmark configurations.

Each initial condition restates the reference's grid-based initialisation for the
corresponding application, evaluated at every allocated point (interior and halos), as the
generated initialisation kernels do over ranges -5..N+5:

  * Sod shock tube             apps/Sod_shock_tube/Sod_shock_tube.py:74-86
  * Taylor-Green vortex        apps/compressible_taylor_green_vortex/compressible_TGV.py:95-117
                               (same fields as apps/taylor_green_vortex/taylor_green_vortex.py:84-100)
  * Kelvin-Helmholtz ensemble  apps/kelvin_helmholtz/kelvin_helmholtz.py:74-89, with the HDF5
                               random perturbation replaced by a seeded sine mode per instance
"""
import math

import numpy as np

from . import abi
from .spec import BlockSpec

RK3_LS_A = (0.0, -5.0 / 9.0, -153.0 / 128.0)    # rk_LS.py:116-118
RK3_LS_B = (1.0 / 3.0, 15.0 / 16.0, 8.0 / 15.0)
RK3_SBLI_NEW = (2.0 / 3.0, 5.0 / 12.0, 3.0 / 5.0)  # rk_sbli.py:75-77 (stage coefficients)
RK3_SBLI_OLD = (1.0 / 4.0, 3.0 / 20.0, 3.0 / 5.0)  # (solution coefficients)
# Three-stage third-order SSP coefficients of the low-storage form (rk_LS.py:102-106, Ruuth
# 2005; the shock-reflection app's RungeKuttaLS(3, formulation='SSP'))
RK3_SSP_A = (0.0, -2.915493957701923, 0.0)
RK3_SSP_B = (0.924574112262461, 0.287712943868770, 0.626538293270800)


def _cons(spec, rho, u, p):
    g = spec.gama
    q = [rho]
    ke = 0.0
    for ui in u:
        q.append(rho * ui)
        ke = ke + ui * ui
    q.append(p / (g - 1.0) + 0.5 * rho * ke)
    return [np.ascontiguousarray(np.broadcast_to(x, spec.shape), dtype=np.float64) for x in q]


def sod(n=400, scheme=abi.SCHEME_WENO5_JS, bc=(abi.BC_ZERO_GRAD, abi.BC_ZERO_GRAD)):
    """1D Sod shock tube on [0,1] with Delta = 1/(N-1); zero-gradient ends unless `bc` names
    other boundary kinds (left, right)."""
    spec = BlockSpec(ndim=1, size=(n,), scheme=scheme, averaging=abi.AVG_SIMPLE,
                     bc=[list(bc)], bc_depth=[[4, 4]],
                     delta=(1.0 / (n - 1),), gama=1.4)
    x = spec.delta[0] * spec.grid_index(0)
    left = x < 0.5
    rho = np.where(left, 1.0, 0.125)
    p = np.where(left, 1.0, 0.1)
    u = np.zeros_like(x, dtype=np.float64)
    return spec, _cons(spec, rho, [u], p)


def tgv(n=64, minf=0.1, scheme=abi.SCHEME_CENTRAL4, averaging=abi.AVG_SIMPLE, viscous=None, sizes=None):
    """3D Taylor-Green vortex on the periodic box [0, 2pi)^3."""
    sizes = tuple(sizes) if sizes is not None else (n, n, n)
    if viscous is None:
        viscous = abi.VISC_CONSTANT if scheme == abi.SCHEME_CENTRAL4 else abi.VISC_SUTHERLAND
    depth = 2 if scheme == abi.SCHEME_CENTRAL4 else 4
    spec = BlockSpec(ndim=3, size=sizes, scheme=scheme, averaging=averaging, viscous=viscous,
                     bc=[[abi.BC_PERIODIC] * 2 for _ in range(3)], bc_depth=[[depth] * 2 for _ in range(3)],
                     delta=tuple(2.0 * math.pi / s for s in sizes), gama=1.4, Minf=minf, Re=1600.0, Pr=0.71,
                     mu_const=1.0, eps=1e-40, teno_ct=1e-6)
    x0 = spec.delta[0] * spec.grid_index(0)
    x1 = spec.delta[1] * spec.grid_index(1)
    x2 = spec.delta[2] * spec.grid_index(2)
    g = spec.gama
    u0 = np.sin(x0) * np.cos(x1) * np.cos(x2)
    u1 = -np.cos(x0) * np.sin(x1) * np.cos(x2)
    u2 = np.zeros_like(u0)
    p = (2.0 + np.cos(2.0 * x2)) * (0.0625 * np.cos(2.0 * x0) + 0.0625 * np.cos(2.0 * x1)) + 1.0 / (minf * minf * g)
    r = g * p * minf * minf
    return spec, _cons(spec, r, [u0, u1, u2], p)


def stretched_line(n, stretch, j=None):
    """Wall-normal coordinate y = -tanh(s (1 - 2 j / (n - 1))) / tanh(s) of the rows j (default
    the interior rows 0..n-1), the generated grid kernel's operation order
    (apps/channel_flow/compressible_TCF_TENO/turbulent_channel.py:178)."""
    j = np.arange(n) if j is None else j
    return -1.0 * np.tanh((1.0 - 2.0 * j / (-1.0 + n)) * stretch) / np.tanh(stretch)


def channel_iso(sizes=(16, 17, 8), twall=1.0, minf=0.5, re=100.0, upper="isothermal", stretch=None):
    """3D channel between isothermal no-slip walls at y = -1 and y = 1 (IsothermalWallBC on both
    y faces, Twall = `twall`), periodic in x on [0, 2pi) and z on [0, 2pi), uniform grid with the
    walls on the first and last points in y (Delta_y = 2 / (N_y - 1)), characteristic LLF TENO5
    (Roe average) with central-4 viscous terms (modified Sutherland law), Minf = 0.5, Re = 100:
    the shock-capturing wall-bounded form of the SBLI apps with the walls of
    apps/channel_flow/compressible_TCF_Central/turbulent_channel.py:118-131.  Initial state: a
    perturbed parabolic profile, u0 = (1 - y^2)(1 + 0.1 sin x cos z), u1 = 0.05 sin x (1 - y^2)^2,
    u2 = 0.05 cos x sin z (1 - y^2), p = (1 + 0.02 cos x cos z) / (gama Minf^2),
    rho = 1 + 0.02 sin x y.  upper = "adiabatic" makes the upper wall an AdiabaticWallBC (the
    alternative upper wall of apps/channel_flow/laminar_2D/laminar_channel.py:104-113).

    stretch = s (e.g. 1.7): the wall-normal grid of apps/channel_flow/compressible_TCF_TENO/
    turbulent_channel.py:170-232, y = -tanh(s (1 - 2 j / (N_y - 1))) / tanh(s) on xi_1 in [0, 1]
    (Delta_1 = 1 / (N_y - 1)), whose metrics D11 / SD111 (osb_ystretch_metrics) the spec carries."""
    n0, n1, n2 = sizes
    spec = BlockSpec(ndim=3, size=sizes, scheme=abi.SCHEME_TENO5, averaging=abi.AVG_ROE,
                     viscous=abi.VISC_SUTHERLAND,
                     bc=[[abi.BC_PERIODIC] * 2,
                         [abi.BC_ISOTHERMAL_WALL, abi.BC_ISOTHERMAL_WALL if upper == "isothermal" else abi.BC_ADIABATIC_WALL],
                         [abi.BC_PERIODIC] * 2],
                     bc_depth=[[4, 4] for _ in range(3)],
                     delta=(2.0 * math.pi / n0, (1.0 if stretch else 2.0) / (n1 - 1), 2.0 * math.pi / n2),
                     gama=1.4, Minf=minf, Re=re,
                     Pr=0.71, mu_const=1.0, eps=1e-40, teno_ct=1e-6,
                     wall_temperature={(1, 0): float(twall), (1, 1): float(twall)} if upper == "isothermal"
                     else {(1, 0): float(twall)})
    x0 = spec.delta[0] * spec.grid_index(0)
    if stretch:
        x1 = stretched_line(n1, stretch, spec.grid_index(1))
        spec.ystretch = abi.ystretch_metrics(stretched_line(n1, stretch), spec.delta[1])
    else:
        x1 = -1.0 + spec.delta[1] * spec.grid_index(1)
    x2 = spec.delta[2] * spec.grid_index(2)
    g = spec.gama
    w = 1.0 - x1 * x1
    u0 = w * (1.0 + 0.1 * np.sin(x0) * np.cos(x2))
    u1 = 0.05 * np.sin(x0) * w * w
    u2 = 0.05 * np.cos(x0) * np.sin(x2) * w
    p = 1.0 / (g * minf * minf) * (1.0 + 0.02 * np.cos(x0) * np.cos(x2))
    r = 1.0 + 0.02 * np.sin(x0) * x1
    return spec, _cons(spec, r, [u0, u1, u2], p)


def channel_tcf(sizes=(16, 17, 8), stretch=1.7):
    """The discretisation and parameters of apps/channel_flow/compressible_TCF_TENO/
    turbulent_channel.py: characteristic LLF TENO6 (Roe average) + central-4 viscous terms with
    the power-law viscosity mu = T^0.7, the constant forcing c = (-1, 0, 0) (-c_i in the momentum
    equations, -c_j u_j in the energy equation), isothermal walls (Twall 1) on the tanh-stretched
    wall-normal grid (xi_1 in [0, 2], stretch 1.7), periodic x on [0, 4 pi) and z on
    [0, 4 pi / 3), Re 190.71, Minf 0.0955, Pr 0.7, TENO_CT 1e-7, and the TENO epsilon 1e-40 that
    the generated code uses (the app's eps = 1e-15 parameter does not reach it: LFTeno fixes the
    value, teno.py:368-371); the initial fields of channel_iso on that grid."""
    n0, n1, n2 = sizes
    spec = BlockSpec(ndim=3, size=sizes, scheme=abi.SCHEME_TENO6, averaging=abi.AVG_ROE,
                     viscous=abi.VISC_POWER_LAW, visc_power=0.7, forcing=(-1.0, 0.0, 0.0),
                     bc=[[abi.BC_PERIODIC] * 2, [abi.BC_ISOTHERMAL_WALL] * 2, [abi.BC_PERIODIC] * 2],
                     bc_depth=[[4, 4] for _ in range(3)],
                     delta=(4.0 * math.pi / n0, 2.0 / (n1 - 1), (4.0 * math.pi / 3.0) / n2),
                     gama=1.4, Minf=0.0955, Re=190.71, Pr=0.7, mu_const=1.0, eps=1e-40, teno_ct=1e-7,
                     wall_temperature={(1, 0): 1.0, (1, 1): 1.0})
    x0 = spec.delta[0] * spec.grid_index(0)
    x1 = stretched_line(n1, stretch, spec.grid_index(1))
    spec.ystretch = abi.ystretch_metrics(stretched_line(n1, stretch), spec.delta[1])
    x2 = spec.delta[2] * spec.grid_index(2)
    g = spec.gama
    w = 1.0 - x1 * x1
    u0 = w * (1.0 + 0.1 * np.sin(x0) * np.cos(x2))
    u1 = 0.05 * np.sin(x0) * w * w
    u2 = 0.05 * np.cos(x0) * np.sin(x2) * w
    p = 1.0 / (g * spec.Minf * spec.Minf) * (1.0 + 0.02 * np.cos(x0) * np.cos(x2))
    r = 1.0 + 0.02 * np.sin(x0) * x1
    return spec, _cons(spec, r, [u0, u1, u2], p)


def duct_inlet(sizes=(20, 17, 8), minf=0.5, re=100.0):
    """The inflow / outflow faces of the SBLI apps (apps/katzer_SBLI/katzer_SBLI.py:131-160) on a
    3D duct x in [0, 4], y in [-1, 1] (walls), z in [0, 2 pi) (periodic): the pressure-extrapolation
    inlet at x = 0, zeroth-order extrapolation at x = 4, isothermal walls (Twall 1) on both y faces;
    characteristic LLF TENO5 (Roe) + central viscous terms (modified Sutherland), Re 100.  Initial
    state (over the whole allocation: the inlet's halos keep it as the inflow)
    u0 = (1 - y^2)(1 + 0.05 sin z), u1 = 0.05 sin x (1 - y^2)^2, u2 = 0.05 cos x sin z (1 - y^2),
    p = (1 + 0.02 cos x cos z) / (gama Minf^2), rho = 1 + 0.02 sin x y.  minf 0.5 takes the
    inlet's subsonic branch, 2 its supersonic one.  The inlet is restated in the oracle only: the
    GPU path refuses this spec."""
    n0, n1, n2 = sizes
    spec = BlockSpec(ndim=3, size=sizes, scheme=abi.SCHEME_TENO5, averaging=abi.AVG_ROE,
                     viscous=abi.VISC_SUTHERLAND,
                     bc=[[abi.BC_INLET_PRESSURE_EXTRAP, abi.BC_EXTRAP0], [abi.BC_ISOTHERMAL_WALL] * 2,
                         [abi.BC_PERIODIC] * 2],
                     bc_depth=[[4, 4] for _ in range(3)],
                     delta=(4.0 / (n0 - 1), 2.0 / (n1 - 1), 2.0 * math.pi / n2), gama=1.4, Minf=minf, Re=re,
                     Pr=0.71, mu_const=1.0, eps=1e-40, teno_ct=1e-6, wall_temperature={(1, 0): 1.0, (1, 1): 1.0})
    x0 = spec.delta[0] * spec.grid_index(0)
    x1 = -1.0 + spec.delta[1] * spec.grid_index(1)
    x2 = spec.delta[2] * spec.grid_index(2)
    g = spec.gama
    w = 1.0 - x1 * x1
    u0 = w * (1.0 + 0.05 * np.sin(x2))
    u1 = 0.05 * np.sin(x0) * w * w
    u2 = 0.05 * np.cos(x0) * np.sin(x2) * w
    p = 1.0 / (g * minf * minf) * (1.0 + 0.02 * np.cos(x0) * np.cos(x2))
    r = 1.0 + 0.02 * np.sin(x0) * x1
    return spec, _cons(spec, r, [u0, u1, u2], p)


def katzer_line(n1, lx1=115.0, by=5.0, j=None):
    """Wall-normal coordinate of the Katzer SBLI grid, Lx1 sinh(by xi_1 / Lx1) / sinh(by) with
    xi_1 = Delta_1 j, Delta_1 = Lx1 / (n1 - 1), in the generated grid kernel's operation order
    (apps/katzer_SBLI/katzer_SBLI.py:185)."""
    j = np.arange(n1) if j is None else j
    d1 = lx1 / (n1 - 1)
    inv = 1.0 / lx1
    return np.sinh(by * inv * d1 * j) / (inv * np.sinh(by))


def katzer(sizes=(24, 17)):
    """The discretisation of apps/katzer_SBLI/katzer_SBLI.py (direct shock-capturing branch) on
    a small block: 2D, WENO5-Z (simple average, LLF) + central viscous terms with Sutherland's
    law (S = SuthT / RefT = 110.4 / 288), Minf 2, Re 950, Pr 0.72, the SSP RK3; x in [0, 400]
    (Delta_0 = 400 / (n0 - 1)) with the pressure-extrapolation inlet at x = 0 and zeroth-order
    extrapolation at x = 400; the sinh-stretched wall-normal grid y in [0, 115] (katzer_line)
    with an isothermal wall (Twall 1.67619431) at y = 0 and the app's Dirichlet shock-generator
    state (post-shock where x0 > 40) over the top plane and its 4 halo layers.  Initial fields
    (the app's similarity solution replaced): w = tanh(y / 5), u0 = w (1 + 0.01 sin(0.05 x)),
    u1 = 0.01 w sin(0.1 x), T = Twall + (1 - Twall) w, p = 1 / (gama Minf^2), rho = gama Minf^2 p / T.
    Sutherland's ratio form and the inlet are restated in the oracle only: the GPU path refuses
    this spec."""
    n0, n1 = sizes
    gama, minf, tw = 1.4, 2.0, 1.67619431
    spec = BlockSpec(ndim=2, size=sizes, scheme=abi.SCHEME_WENO5_Z, averaging=abi.AVG_SIMPLE,
                     viscous=abi.VISC_SUTHERLAND_RATIO, sutherland_s=110.4 * (1.0 / 288.0),
                     bc=[[abi.BC_INLET_PRESSURE_EXTRAP, abi.BC_EXTRAP0], [abi.BC_ISOTHERMAL_WALL, abi.BC_DIRICHLET]],
                     bc_depth=[[4, 4], [4, 4]], delta=(400.0 / (n0 - 1), 115.0 / (n1 - 1)), gama=gama, Minf=minf,
                     Re=950.0, Pr=0.72, eps=1e-40, wall_temperature={(1, 0): tw})
    x0 = spec.delta[0] * spec.grid_index(0)
    x1 = katzer_line(n1, j=spec.grid_index(1))
    spec.ystretch = abi.ystretch_metrics(katzer_line(n1), spec.delta[1])
    w = np.tanh(x1 / 5.0)
    u0 = w * (1.0 + 0.01 * np.sin(0.05 * x0))
    u1 = 0.01 * w * np.sin(0.1 * x0)
    T = tw + (1.0 - tw) * w
    p = 1.0 / (gama * minf * minf) + 0.0 * T
    r = gama * minf * minf * p / T
    q = _cons(spec, r, [u0, u1], p)
    h = spec.halo
    x = spec.delta[0] * np.arange(-h, n0 + h, dtype=np.float64)
    post = x > 40.0
    top_row = [np.where(post, 1.129734572, 1.00000596004), np.where(post, 1.0921171, 1.00000268202),
               np.where(post, -0.058866065, 0.00565001630205), np.where(post, 1.0590824, 0.94644428042)]
    dep = spec.bc_depth[1][1]
    top = np.empty((4, dep + 1, n0 + 2 * h))
    for v in range(4):
        top[v] = top_row[v][None, :]
    spec.dirichlet = {(1, 1): top}
    return spec, q


def tgv_filtered(n=128, sizes=None, ducros=0.05):
    """The supersonic TGV of the reference's Central4-WENO5 benchmark
    (apps/performance_benchmark/Central4-WENO5; the central branch of
    apps/compressible_taylor_green_vortex/compressible_TGV.py): M = 1.25, Re = 1600, central-4
    KGP split convective terms, modified Sutherland viscosity, the non-linear WENO3-Z filter
    after every step with Ducros_check = Ducros_select = `ducros`; the benchmark's time step is
    0.00084625 * 256 / n (``filtered_dt``)."""
    spec, q = tgv(n, minf=1.25, scheme=abi.SCHEME_CENTRAL4, viscous=abi.VISC_SUTHERLAND, sizes=sizes)
    spec.split_form = abi.SPLIT_KGP
    spec.filter = abi.FILTER_WENO3
    spec.ducros_check = ducros
    spec.ducros_select = ducros
    return spec, q


def tgv_tvd(n=128, sizes=None, kappa=1.25):
    """The supersonic TGV of the central branch of
    apps/compressible_taylor_green_vortex/compressible_TGV.py with its TVD option
    (``TVD = True``): M = 1.25, Re = 1600, central-4 KGP split convective terms, modified
    Sutherland viscosity, periodic exchange of depth 2 after every stage, and the non-linear
    characteristic TVD filter (filters/TVD_filter.py) after every step with strength
    kappa_TVD = `kappa` (1.25 in apps/turbulent_counter_flow)."""
    spec, q = tgv(n, minf=1.25, scheme=abi.SCHEME_CENTRAL4, viscous=abi.VISC_SUTHERLAND, sizes=sizes)
    spec.split_form = abi.SPLIT_KGP
    spec.filter = abi.FILTER_TVD
    spec.tvd_kappa = kappa
    spec.bc_depth = [[2, 2] for _ in range(3)]
    return spec, q


def filtered_dt(n):
    """Time step of the Central4-WENO5 benchmark's strong-scaling mode (opensbli.cpp:63)."""
    return 0.00084625 * 256 / n


def kh(n=128, amp=1.0, phase=0.0, sizes=None, scheme=abi.SCHEME_WENO5_Z, averaging=abi.AVG_ROE):
    """2D Kelvin-Helmholtz on the periodic unit square (Delta = 1/N)."""
    sizes = tuple(sizes) if sizes is not None else (n, n)
    spec = BlockSpec(ndim=2, size=sizes, scheme=scheme, averaging=averaging,
                     bc=[[abi.BC_PERIODIC] * 2 for _ in range(2)], bc_depth=[[4, 4], [4, 4]],
                     delta=(1.0 / sizes[0], 1.0 / sizes[1]), gama=1.4)
    x0 = spec.delta[0] * spec.grid_index(0)
    x1 = spec.delta[1] * spec.grid_index(1)
    band = np.abs(-0.5 + x1) < 0.25
    d = np.where(band, 2.0, 1.0)
    u0 = np.where(band, -0.5, 0.5)
    u1 = 0.01 * amp * np.sin(4.0 * math.pi * x0 + phase)
    p = 2.5
    rho = np.broadcast_to(d, spec.shape)
    return spec, _cons(spec, rho, [np.broadcast_to(u0, spec.shape), np.broadcast_to(u1, spec.shape)], p)


KH_SIZES = (128, 192, 256, 384, 512)


def kh_ensemble(count=64, seed=0, sizes=KH_SIZES):
    """Seeded ensemble of Kelvin-Helmholtz instances of uneven sizes: size, amplitude and
    phase per instance come from numpy.random.default_rng(seed)."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        n = int(rng.choice(sizes))
        amp = float(rng.uniform(0.5, 1.5))
        phase = float(rng.uniform(0.0, 2.0 * math.pi))
        out.append(kh(n=n, amp=amp, phase=phase))
    return out


def cfl_dt(spec, q, cfl):
    """CFL time step dt = cfl / max_points sum_d (|u_d| + a)/Delta_d, in FP64 on the host
    (the reference has no CFL reduction; this is the formula the configs state)."""
    sl = spec.interior()
    rho = q[0][sl]
    g = spec.gama
    ke = 0.0
    us = []
    for d in range(spec.ndim):
        u = q[1 + d][sl] / rho
        us.append(u)
        ke = ke + u * u
    p = (g - 1.0) * (q[-1][sl] - 0.5 * rho * ke)
    a = np.sqrt(g * p / rho)
    s = 0.0
    for d in range(spec.ndim):
        s = s + (np.abs(us[d]) + a) / spec.delta[d]
    return float(cfl / np.max(s))


# ---------------------------------------------------------------------------------------
# Curvilinear blocks.  The metric arrays follow the layout of osb_block_desc.metric:
# index 3*d + i holds D_di = d xi_d / d x_i, index 9 holds det J = det(d x / d xi).

def _d1_central4(f, axis, inv_delta):
    """4th-order central first derivative along a numpy axis, the operator order of the
    generated metric kernel ((-2/3 f[-1] - 1/12 f[+2]) + 1/12 f[-2] + 2/3 f[+1]) * 1/Delta;
    the outer two layers are left at zero."""
    out = np.zeros_like(f)
    n = f.shape[axis]

    def sl(o):
        s = [slice(None)] * f.ndim
        s[axis] = slice(2 + o, n - 2 + o)
        return tuple(s)
    out[sl(0)] = ((-(2.0 / 3.0) * f[sl(-1)] - (1.0 / 12.0) * f[sl(2)]) + (1.0 / 12.0) * f[sl(-2)]
                  + (2.0 / 3.0) * f[sl(1)]) * inv_delta
    return out


def _periodic_fill(spec, a, depth):
    """Periodic halo fill of one OPS-layout array, direction by direction, over the full
    transverse extent (the order of the generated halo exchanges)."""
    h = spec.halo
    for d in range(spec.ndim):
        ax = spec.ndim - 1 - d
        n = spec.size[d]
        lo_dst = [slice(None)] * spec.ndim
        lo_src = [slice(None)] * spec.ndim
        hi_dst = [slice(None)] * spec.ndim
        hi_src = [slice(None)] * spec.ndim
        lo_dst[ax] = slice(h - depth, h)
        lo_src[ax] = slice(h + n - depth, h + n)
        hi_dst[ax] = slice(h + n, h + n + depth)
        hi_src[ax] = slice(h, h + depth)
        a[tuple(lo_dst)] = a[tuple(lo_src)]
        a[tuple(hi_dst)] = a[tuple(hi_src)]


def metrics_central4(spec, x, periodic_from_interior=False, extended=False):
    """Metric arrays of a block from its grid coordinates x[0..ndim-1] (OPS layout, known at
    every allocated point), with 4th-order central derivatives (the reference's
    MetricsEquation with central differences, opensbli/equation_types/metric.py).

    periodic_from_interior=True evaluates them on the interior only and fills the halos by a
    depth-5 periodic exchange, as the generated solver of a periodic curvilinear block does.
    extended=True takes coordinates on the allocation grown by two points on every side and
    evaluates the metrics at every allocated point.  Otherwise they are evaluated wherever the
    stencil fits and the outer two halo layers repeat the nearest evaluated layer."""
    nd = spec.ndim
    J = [[_d1_central4(x[i], nd - 1 - j, 1.0 / spec.delta[j]) for j in range(nd)] for i in range(nd)]
    met = [None] * 10
    if nd == 2:
        det = J[0][0] * J[1][1] - J[0][1] * J[1][0]
        with np.errstate(divide="ignore", invalid="ignore"):
            met[0] = J[1][1] / det
            met[1] = -J[0][1] / det
            met[3] = -J[1][0] / det
            met[4] = J[0][0] / det
        met[9] = det
    else:
        M = np.stack([np.stack(r, axis=-1) for r in J], axis=-2)  # [..., i, j] = d x_i / d xi_j
        det = np.linalg.det(M)
        good = det != 0.0
        inv = np.zeros_like(M)
        inv[good] = np.linalg.inv(M[good])  # [..., d, i] = d xi_d / d x_i
        for d in range(3):
            for i in range(3):
                met[3 * d + i] = np.ascontiguousarray(inv[..., d, i])
        met[9] = det
    h = spec.halo
    for k in range(10):
        if met[k] is None:
            continue
        a = np.ascontiguousarray(met[k])
        if extended:
            a = a[tuple(slice(2, n - 2) for n in a.shape)]
        elif periodic_from_interior:
            b = np.zeros_like(a)
            b[spec.interior()] = a[spec.interior()]
            _periodic_fill(spec, b, h)
            a = b
        else:
            core = tuple(slice(2, s - 2) for s in a.shape)
            pad = [(2, 2)] * a.ndim
            a = np.pad(a[core], pad, mode="edge")
        met[k] = np.ascontiguousarray(a, dtype=np.float64)
    return met


def wave_2d_coords(spec):
    """Grid coordinates of the wavy 2D mesh of curvilinear_wave_2d at every allocated point."""
    i = spec.grid_index(0).astype(np.float64)
    j = spec.grid_index(1).astype(np.float64)
    d0, d1 = spec.delta[0], spec.delta[1]
    x0 = np.broadcast_to(0.04 * np.sin(3 * math.pi * d1 * j) + d0 * i, spec.shape).copy()
    x1 = np.broadcast_to(0.04 * np.sin(3 * math.pi * d0 * i) + d1 * j, spec.shape).copy()
    return x0, x1


def curvilinear_wave_2d(n=128, scheme=abi.SCHEME_WENO5_Z, averaging=abi.AVG_ROE):
    """Density wave on a periodic wavy 2D mesh (the reference's curvilinear Euler verification
    case, tests/verification_apps/euler_wave_curvilinear): Delta = 2/N,
    x0 = i Delta + 0.04 sin(3 pi j Delta), x1 = j Delta + 0.04 sin(3 pi i Delta),
    rho = 1 + 0.2 sin(pi (x0 + x1)), u = (1, -0.5), p = 1; metrics from 4th-order central
    differences on the interior, exchanged periodically.  Returns (spec, state, metrics)."""
    spec = BlockSpec(ndim=2, size=(n, n), scheme=scheme, averaging=averaging,
                     bc=[[abi.BC_PERIODIC] * 2 for _ in range(2)], bc_depth=[[4, 4], [4, 4]],
                     delta=(2.0 / n, 2.0 / n), gama=1.4, curvilinear=True)
    x0, x1 = wave_2d_coords(spec)
    rho = 1.0 + 0.2 * np.sin(math.pi * (x0 + x1))
    q = _cons(spec, rho, [np.full(spec.shape, 1.0), np.full(spec.shape, -0.5)], 1.0)
    return spec, q, metrics_central4(spec, [x0, x1], periodic_from_interior=True)


def wave_3d_coords(spec, amp=0.05):
    """Grid coordinates of the periodic wavy 3D mesh of curvilinear_wave_3d at every allocated
    point: x_i = eta_i + amp sin(2 pi eta_j) sin(2 pi eta_k), (i, j, k) cyclic, eta_d = index_d
    Delta_d."""
    eta = [spec.delta[d] * spec.grid_index(d).astype(np.float64) for d in range(3)]
    out = []
    for i in range(3):
        j, k = (i + 1) % 3, (i + 2) % 3
        x = eta[i] + amp * np.sin(2.0 * math.pi * eta[j]) * np.sin(2.0 * math.pi * eta[k])
        out.append(np.ascontiguousarray(np.broadcast_to(x, spec.shape)))
    return out


def curvilinear_wave_3d(sizes=(16, 12, 10), scheme=abi.SCHEME_TENO5, averaging=abi.AVG_ROE, minf=0.7):
    """Euler on a periodic wavy 3D mesh over the unit box (Delta_d = 1/N_d): coordinates
    wave_3d_coords, rho = 1 + 0.1 sin(2 pi (x0 + x1 + x2)), u = (0.7, -0.3, 0.2),
    p = 1/(gama Minf^2) + 0.1 sin(2 pi (x0 - x1)); metrics from 4th-order central differences on
    the interior, exchanged periodically -- the single-block problem the generated reference case
    curv3d_teno5 solves.  Returns (spec, state, metrics, coordinates)."""
    spec = BlockSpec(ndim=3, size=tuple(sizes), scheme=scheme, averaging=averaging, viscous=abi.VISC_NONE,
                     bc=[[abi.BC_PERIODIC] * 2 for _ in range(3)], bc_depth=[[4, 4] for _ in range(3)],
                     delta=tuple(1.0 / n for n in sizes), gama=1.4, Minf=minf, curvilinear=True)
    x = wave_3d_coords(spec)
    g = spec.gama
    rho = 1.0 + 0.1 * np.sin(2.0 * math.pi * (x[0] + x[1] + x[2]))
    p = 1.0 / (g * minf * minf) + 0.1 * np.sin(2.0 * math.pi * (x[0] - x[1]))
    u = [np.full(spec.shape, c) for c in (0.7, -0.3, 0.2)]
    q = _cons(spec, rho, u, p)
    return spec, q, metrics_central4(spec, x, periodic_from_interior=True), x


def shock_reflection(n0=457, n1=255, sizes=None, flux_type=abi.FLUX_LLF, back_pressure=None):
    """2D inviscid oblique-shock reflection of apps/inviscid_shock_reflection/inviscid_shock.py
    on a 350 x 115 box (Delta = 350/(n0-1), 115/(n1-1)), M = 2, gama = 1.4, WENO5-Z (simple
    average, LLF): uniform free stream (rho = 1, u = (1, 0), p = 1/(gama M^2)); Dirichlet inlet
    (free stream) on the left over the boundary plane and 3 halo layers, zeroth-order
    extrapolation on the right, symmetry (inviscid wall) at the bottom, Dirichlet at the top over
    the plane and 4 halo layers with the post-shock state (rho 1.129734572, u 0.9667023804242755,
    -0.052106102140246795, p 0.211869) from x = 40 and the free stream (p 0.178571) before it --
    values, literals and operation order of the generated boundary and initialisation kernels.
    flux_type = abi.FLUX_HLLC_LM selects the app's own HLLC-LM flux, back_pressure a
    PressureOutletBC in place of the extrapolation outlet."""
    if sizes is not None:
        n0, n1 = sizes
    gama, minf = 1.4, 2.0
    spec = BlockSpec(ndim=2, size=(n0, n1), scheme=abi.SCHEME_WENO5_Z, averaging=abi.AVG_SIMPLE,
                     bc=[[abi.BC_DIRICHLET, abi.BC_EXTRAP0], [abi.BC_SYMMETRY, abi.BC_DIRICHLET]],
                     bc_depth=[[3, 4], [4, 4]], delta=(350.0 / (n0 - 1), 115.0 / (n1 - 1)), gama=gama, Minf=minf,
                     flux_type=flux_type)
    inv_gm1 = 1.0 / (-1 + gama)
    p_inf = 1.0 * (1.0 / gama) * (minf ** -2.0)

    def cons(d, u0, u1, p):
        return [d, d * u0, d * u1, p * inv_gm1 + 0.5 * d * ((u0 * u0) + (u1 * u1))]

    free = cons(1.0, 1.0, 0.0, p_inf)
    q = [np.full(spec.shape, v) for v in free]
    h = spec.halo
    # left inlet: plane x = 0 and 3 halo layers, every allocated y
    dep0 = spec.bc_depth[0][0]
    left = np.empty((4, dep0 + 1, n1 + 2 * h))
    for v in range(4):
        left[v] = free[v]
    # top: plane y = n1-1 and 4 halo layers, every allocated x; x = Delta0 * i
    dep1 = spec.bc_depth[1][1]
    x = spec.delta[0] * np.arange(-h, n0 + h, dtype=np.float64)
    pre = x < 40.0
    d = np.where(pre, 1.0, 1.129734572)
    u0 = np.where(pre, 1.0, 0.9667023804242755)
    u1 = np.where(pre, 0.0, -0.052106102140246795)
    p = np.where(pre, 0.178571, 0.211869)
    top_row = cons(d, u0, u1, p)
    top = np.empty((4, dep1 + 1, n0 + 2 * h))
    for v in range(4):
        top[v] = top_row[v][None, :]
    spec.dirichlet = {(0, 0): left, (1, 1): top}
    if back_pressure is not None:
        spec.bc[0][1] = abi.BC_PRESSURE_OUTLET
        spec.back_pressure = {(0, 1): float(back_pressure)}
    return spec, q


# ---------------------------------------------------------------------------------------
# Multi-block topologies

def flipped_pair_2d(sizes=(24, 20)):
    """Two 2D Euler blocks (WENO5-Z, simple average) joined along x by two flipped interfaces --
    block 0's low-x face to block 1's low-x face and the two high-x faces (InterfaceBC with the
    match flag set, as a C-mesh wake cut) -- and periodic in y (depth 4 everywhere), with a
    different smooth state on each block over x0 = i / N0, x1 = j / N1: the problem of the
    generated multi-block reference case mb2_flip.  Returns [(spec, state)] for blocks 0 and 1."""
    forms = [(lambda x0, x1: 1.0 + 0.2 * np.sin(2 * math.pi * (x0 + x1)),
              lambda x0, x1: 0.4 + 0.1 * np.cos(2 * math.pi * x1),
              lambda x0, x1: -0.2 + 0.1 * np.sin(2 * math.pi * x0),
              lambda x0, x1: 1.0 + 0.1 * np.cos(2 * math.pi * (x0 - x1))),
             (lambda x0, x1: 1.1 + 0.15 * np.cos(2 * math.pi * (x0 - 2 * x1)),
              lambda x0, x1: -0.3 + 0.1 * np.sin(2 * math.pi * (x0 + x1)),
              lambda x0, x1: 0.25 + 0.1 * np.cos(2 * math.pi * x0),
              lambda x0, x1: 0.9 + 0.1 * np.sin(2 * math.pi * x1))]
    out = []
    for b in range(2):
        o = 1 - b
        spec = BlockSpec(ndim=2, size=tuple(sizes), scheme=abi.SCHEME_WENO5_Z, averaging=abi.AVG_SIMPLE,
                         bc=[[abi.BC_INTERFACE, abi.BC_INTERFACE], [abi.BC_PERIODIC, abi.BC_PERIODIC]],
                         bc_depth=[[4, 4], [4, 4]], iface=[[(o, 0, 0, 1), (o, 0, 1, 1)], [None, None]],
                         delta=(1.0 / sizes[0], 1.0 / sizes[1]), gama=1.4)
        x0 = spec.delta[0] * spec.grid_index(0)
        x1 = spec.delta[1] * spec.grid_index(1)
        d, u0, u1, p = (f(x0, x1) for f in forms[b])
        out.append((spec, _cons(spec, d, [u0, u1], p)))
    return out


def split_block(spec, state, cuts, d=0, metrics=None):
    """Split one block along direction d at the interior indices `cuts` into blocks joined by
    interfaces (periodic faces along d become an interface between the last and the first
    piece).  Returns [(spec, state[, metrics])] in OPS layout; each piece's arrays are the
    matching window of the original allocation, halos included."""
    h = spec.halo
    edges = [0] + list(cuts) + [spec.size[d]]
    nb = len(edges) - 1
    ax = spec.ndim - 1 - d
    out = []
    for b in range(nb):
        lo, hi = edges[b], edges[b + 1]
        size = list(spec.size)
        size[d] = hi - lo
        bc = [list(x) for x in spec.bc]
        iface = [[None, None] for _ in range(spec.ndim)]
        if spec.iface is not None:
            iface = [list(x) for x in spec.iface]
        periodic = spec.bc[d][0] == abi.BC_PERIODIC
        if b > 0 or periodic:
            bc[d][0] = abi.BC_INTERFACE
            iface[d][0] = ((b - 1) % nb, d, 1, 0)
        if b < nb - 1 or periodic:
            bc[d][1] = abi.BC_INTERFACE
            iface[d][1] = ((b + 1) % nb, d, 0, 0)
        ps = BlockSpec(**{**spec.__dict__, "size": tuple(size), "bc": bc, "iface": iface})
        win = [slice(None)] * spec.ndim
        win[ax] = slice(lo, hi + 2 * h)
        win = tuple(win)
        st = [np.ascontiguousarray(a[win]) for a in state]
        if metrics is None:
            out.append((ps, st))
        else:
            out.append((ps, st, [None if m is None else np.ascontiguousarray(m[win]) for m in metrics]))
    return out


MB_SIZES = {"A": (512, 256, 32), "B": (384, 256, 32), "C": (512, 192, 32), "D": (256, 256, 32)}


def curvilinear_multiblock_3d(sizes=None, seed=0, amp=0.05, mach=0.7, pulse=1e-2, sigma=0.1,
                              scheme=abi.SCHEME_TENO5, averaging=abi.AVG_ROE):
    """Four curvilinear 3D Euler blocks joined by interfaces (blocks A, B, C, D in that order):
    A, B, D form a chain along x (D's high-x face wraps to A), C sits on A's high-y face and
    wraps to A's low-y face, B and D are periodic in y, C in x, every block in z.  The grid is
    uniform in index space with Delta = 1/nz,
        x = xi   + amp sin(2 pi eta / L_eta) sin(2 pi zeta / L_zeta)
        y = eta  + amp sin(2 pi xi / L_xi)   sin(2 pi zeta / L_zeta)
        z = zeta + amp sin(2 pi xi / L_xi)   sin(2 pi eta / L_eta)
    with the periods chosen so that every periodic wrap and interface meets a continuous mesh
    (L_xi: gcd of the x chain and C's x length, L_eta: gcd of the A-C chain and B's y length,
    L_zeta: nz).  Metrics come from 4th-order central differences of the analytic mesh at every
    allocated point.  Initial state: uniform flow at Mach `mach` along x (rho = 1, p = 1/gama,
    so a = 1) plus a Gaussian pulse g = exp(-r^2 / (2 sigma^2)) of relative amplitude `pulse`
    in density and gama * pulse in pressure (isentropic to first order), centred at a seeded
    point of block A.  Returns [(spec, state, metrics)] for A, B, C, D."""
    sizes = dict(MB_SIZES if sizes is None else sizes)
    A, B, C, D = (sizes[k] for k in "ABCD")
    nz = A[2]
    assert all(s[2] == nz for s in (A, B, C, D)) and B[1] == A[1] and D[1] == A[1] and C[0] == A[0]
    dl = 1.0 / nz
    Lxi = math.gcd(A[0] + B[0] + D[0], C[0]) * dl
    Leta = math.gcd(A[1] + C[1], B[1]) * dl
    Lzeta = nz * dl
    g = 1.4
    P, I = abi.BC_PERIODIC, abi.BC_INTERFACE
    # origin (in points) and faces of every block
    layout = {
        "A": ((0, 0, 0), [[I, I], [I, I], [P, P]], [[(3, 0, 1, 0), (1, 0, 0, 0)], [(2, 1, 1, 0), (2, 1, 0, 0)], [None, None]]),
        "B": ((A[0], 0, 0), [[I, I], [P, P], [P, P]], [[(0, 0, 1, 0), (3, 0, 0, 0)], [None, None], [None, None]]),
        "C": ((0, A[1], 0), [[P, P], [I, I], [P, P]], [[None, None], [(0, 1, 1, 0), (0, 1, 0, 0)], [None, None]]),
        "D": ((A[0] + B[0], 0, 0), [[I, I], [P, P], [P, P]], [[(1, 0, 1, 0), (0, 0, 0, 0)], [None, None], [None, None]]),
    }
    rng = np.random.default_rng(seed)
    centre = [rng.uniform(0.25, 0.75) * A[d] * dl for d in range(3)]
    out = []
    for name in "ABCD":
        size = sizes[name]
        org, bc, iface = layout[name]
        spec = BlockSpec(ndim=3, size=size, scheme=scheme, averaging=averaging, viscous=abi.VISC_NONE,
                         bc=bc, bc_depth=[[4, 4] for _ in range(3)], iface=iface, delta=(dl, dl, dl), gama=g,
                         curvilinear=True)
        # index coordinates on the allocation grown by 2 (for the metric stencil)
        grids = []
        for d in range(3):
            n = size[d] + 2 * spec.halo + 4
            idx = (np.arange(n) - spec.halo - 2 + org[d]) * dl
            shp = [1, 1, 1]
            shp[2 - d] = n
            grids.append(idx.reshape(shp))
        xi, eta, zeta = grids
        ext_shape = tuple(s + 4 for s in spec.shape)
        two_pi = 2.0 * math.pi
        x0 = np.broadcast_to(xi + amp * np.sin(two_pi * eta / Leta) * np.sin(two_pi * zeta / Lzeta), ext_shape)
        x1 = np.broadcast_to(eta + amp * np.sin(two_pi * xi / Lxi) * np.sin(two_pi * zeta / Lzeta), ext_shape)
        x2 = np.broadcast_to(zeta + amp * np.sin(two_pi * xi / Lxi) * np.sin(two_pi * eta / Leta), ext_shape)
        met = metrics_central4(spec, [np.ascontiguousarray(x0), np.ascontiguousarray(x1), np.ascontiguousarray(x2)],
                               extended=True)
        core = tuple(slice(2, n - 2) for n in ext_shape)
        r2 = (x0[core] - centre[0]) ** 2 + (x1[core] - centre[1]) ** 2 + (x2[core] - centre[2]) ** 2
        gs = np.exp(-r2 / (2.0 * sigma * sigma))
        rho = 1.0 + pulse * gs
        p = (1.0 / g) * (1.0 + g * pulse * gs)
        zero = np.zeros(spec.shape)
        q = _cons(spec, rho, [np.full(spec.shape, mach), zero, zero], p)
        out.append((spec, q, met))
    return out


def multiblock_cfl_dt(blocks, cfl):
    """CFL time step over curvilinear blocks: cfl / max sum_d (|U_d| + a |D_d|) with
    U_d = D_d . u (physical speeds mapped to index space), FP64 on the host."""
    worst = 0.0
    for spec, q, met in blocks:
        sl = spec.interior()
        rho = q[0][sl]
        u = [q[1 + i][sl] / rho for i in range(spec.ndim)]
        ke = sum(ui * ui for ui in u)
        p = (spec.gama - 1.0) * (q[-1][sl] - 0.5 * rho * ke)
        a = np.sqrt(spec.gama * p / rho)
        s = 0.0
        for d in range(spec.ndim):
            Dd = [met[3 * d + i][sl] for i in range(spec.ndim)]
            U = sum(Dd[i] * u[i] for i in range(spec.ndim))
            nrm = np.sqrt(sum(x * x for x in Dd))
            s = s + (np.abs(U) + a * nrm) / spec.delta[d]
        worst = max(worst, float(np.max(s)))
    return cfl / worst
