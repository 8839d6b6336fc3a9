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


def _cons(spec, rho, u, p):
    g = spec.gama
    q = [rho]
    ke = 0.0
    for ui in u:
        q.append(rho * ui)
        ke = ke + ui * ui
    q.append(p / (g - 1.0) + 0.5 * rho * ke)
    return [np.ascontiguousarray(np.broadcast_to(x, spec.shape), dtype=np.float64) for x in q]


def sod(n=400, scheme=abi.SCHEME_WENO5_JS):
    """1D Sod shock tube on [0,1] with Delta = 1/(N-1), zero-gradient ends."""
    spec = BlockSpec(ndim=1, size=(n,), scheme=scheme, averaging=abi.AVG_SIMPLE,
                     bc=[[abi.BC_ZERO_GRAD, abi.BC_ZERO_GRAD]], bc_depth=[[4, 4]],
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
