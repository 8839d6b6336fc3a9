"""Block specifications and OPS-layout array helpers.

A ``BlockSpec`` is the Python form of ``osb_block_desc`` (include/osb_gb300.h) minus the
array pointers.  ``opensbli_gb300.backend`` builds one per OpenSBLI ``SimulationBlock`` (by
walking the reference's scheme / boundary / constant objects) or takes them directly from a
caller that does not use the OpenSBLI front end.
"""
from dataclasses import dataclass, field
from typing import List, Optional, Tuple

import numpy as np

from . import abi

HALO = 5


@dataclass
class BlockSpec:
    ndim: int
    size: Tuple[int, ...]
    scheme: int
    averaging: int = abi.AVG_SIMPLE
    viscous: int = abi.VISC_NONE
    bc: List[List[int]] = None
    bc_depth: List[List[int]] = None
    iface: Optional[list] = None
    gama: float = 1.4
    Minf: float = 1.0
    Re: float = 1.0
    Pr: float = 0.71
    mu_const: float = 1.0
    eps: float = 1e-40
    teno_ct: float = 1e-6
    shock_filter_control: float = 1.0
    delta: Tuple[float, ...] = (1.0, 1.0, 1.0)
    halo: int = HALO
    split_form: int = abi.SPLIT_FEIEREISEN
    filter: int = abi.FILTER_NONE
    ducros_check: float = 0.05
    ducros_select: float = 0.05
    tvd_kappa: float = 1.0
    # Dirichlet faces: {(direction, side): array [v][layer][t]} of the values on the boundary
    # plane and its bc_depth halo layers (osb_block_desc.dirichlet)
    dirichlet: dict = None
    flux_type: int = abi.FLUX_LLF
    # pressure-outlet faces: {(direction, side): back pressure}
    back_pressure: dict = None
    # isothermal-wall faces: {(direction, side): wall temperature Twall}
    wall_temperature: dict = None
    # a curvilinear block: its metric arrays (osb_block_desc.metric) must be supplied; a
    # curvilinear block without them is refused instead of being run as a Cartesian one
    curvilinear: bool = False
    # a stretched wall-normal grid: (D11, SD111) of the interior rows (osb_block_desc.ystretch,
    # abi.ystretch_metrics); delta[1] is then the spacing of xi_1
    ystretch: tuple = None
    # OSB_VISC_POWER_LAW exponent, and the constant source terms c_j of the channel apps
    # (osb_block_desc.visc_power / forcing)
    visc_power: float = 0.0
    forcing: tuple = None
    # OSB_VISC_SUTHERLAND_RATIO: S = SuthT / RefT
    sutherland_s: float = 0.0

    def __post_init__(self):
        self.size = tuple(int(s) for s in self.size)
        if self.bc is None:
            self.bc = [[abi.BC_PERIODIC, abi.BC_PERIODIC] for _ in range(self.ndim)]
        if self.bc_depth is None:
            self.bc_depth = [[4, 4] for _ in range(self.ndim)]
        if len(self.delta) < 3:
            self.delta = tuple(self.delta) + (1.0,) * (3 - len(self.delta))

    @property
    def nvars(self):
        return self.ndim + 2

    @property
    def shape(self):
        """numpy shape of one OPS-layout array (slowest first)."""
        ext = [self.size[d] + 2 * self.halo for d in range(self.ndim)]
        return tuple(reversed(ext))

    @property
    def npoints(self):
        n = 1
        for d in range(self.ndim):
            n *= self.size[d]
        return n

    def interior(self):
        """Slice tuple selecting the interior of an OPS-layout array."""
        h = self.halo
        return tuple(slice(h, h + self.size[d]) for d in reversed(range(self.ndim)))

    def grid_index(self, d):
        """Global index (OPS ``idx``) of every allocated point along direction d, broadcastable."""
        n = self.size[d] + 2 * self.halo
        idx = np.arange(n) - self.halo
        shp = [1] * self.ndim
        shp[self.ndim - 1 - d] = n
        return idx.reshape(shp)

    # ---- serialisation (the backend's plan files): scalars and lists as plain values, the
    # Dirichlet face arrays separately
    _SCALARS = ("ndim", "scheme", "averaging", "viscous", "gama", "Minf", "Re", "Pr", "mu_const", "eps", "teno_ct",
                "shock_filter_control", "halo", "split_form", "filter", "ducros_check", "ducros_select", "tvd_kappa",
                "flux_type", "curvilinear")

    def to_record(self):
        """(dict of plain values, {name: array}) that from_record turns back into this spec."""
        rec = {k: getattr(self, k) for k in self._SCALARS}
        rec["curvilinear"] = bool(self.curvilinear)
        rec["size"] = list(self.size)
        rec["delta"] = [float(x) for x in self.delta]
        rec["bc"] = [list(map(int, r)) for r in self.bc]
        rec["bc_depth"] = [list(map(int, r)) for r in self.bc_depth]
        rec["iface"] = None if self.iface is None else [[None if f is None else list(map(int, f)) for f in r]
                                                        for r in self.iface]
        rec["back_pressure"] = None if not self.back_pressure else [[d, s, float(v)] for (d, s), v in
                                                                     sorted(self.back_pressure.items())]
        if self.visc_power:  # (absent otherwise, like the wall temperatures)
            rec["visc_power"] = float(self.visc_power)
        if self.forcing and any(self.forcing):
            rec["forcing"] = [float(c) for c in self.forcing]
        if self.sutherland_s:
            rec["sutherland_s"] = float(self.sutherland_s)
        if self.wall_temperature:  # (absent otherwise: records of blocks without walls are unchanged)
            rec["wall_temperature"] = [[d, s, float(v)] for (d, s), v in sorted(self.wall_temperature.items())]
        arrays = {"dirichlet_%d_%d" % k: np.ascontiguousarray(a) for k, a in (self.dirichlet or {}).items()}
        if self.ystretch is not None:
            arrays["ystretch_d11"], arrays["ystretch_sd111"] = (np.ascontiguousarray(a) for a in self.ystretch)
        return rec, arrays

    @classmethod
    def from_record(cls, rec, arrays=None):
        kw = {k: rec[k] for k in cls._SCALARS if k in rec}
        kw["size"] = tuple(rec["size"])
        kw["delta"] = tuple(rec["delta"])
        kw["bc"] = [list(r) for r in rec["bc"]]
        kw["bc_depth"] = [list(r) for r in rec["bc_depth"]]
        if rec.get("iface") is not None:
            kw["iface"] = [[None if f is None else tuple(f) for f in r] for r in rec["iface"]]
        if rec.get("back_pressure"):
            kw["back_pressure"] = {(int(d), int(s)): float(v) for d, s, v in rec["back_pressure"]}
        if rec.get("wall_temperature"):
            kw["wall_temperature"] = {(int(d), int(s)): float(v) for d, s, v in rec["wall_temperature"]}
        if rec.get("visc_power"):
            kw["visc_power"] = float(rec["visc_power"])
        if rec.get("forcing"):
            kw["forcing"] = tuple(float(c) for c in rec["forcing"])
        if rec.get("sutherland_s"):
            kw["sutherland_s"] = float(rec["sutherland_s"])
        dirichlet = {}
        for name, a in (arrays or {}).items():
            if name.startswith("dirichlet_"):
                _, d, s = name.split("_")
                dirichlet[(int(d), int(s))] = np.asarray(a, dtype=np.float64)
        if dirichlet:
            kw["dirichlet"] = dirichlet
        if arrays is not None and "ystretch_d11" in arrays:
            kw["ystretch"] = (np.asarray(arrays["ystretch_d11"], dtype=np.float64),
                              np.asarray(arrays["ystretch_sd111"], dtype=np.float64))
        return cls(**kw)

    def same_discretisation(self, other):
        return (self.ndim, self.scheme, self.averaging, self.viscous, self.split_form, self.filter,
                self.flux_type) == (other.ndim, other.scheme, other.averaging, other.viscous, other.split_form,
                                    other.filter, other.flux_type)


def empty_state(spec):
    return [np.zeros(spec.shape, dtype=np.float64) for _ in range(spec.nvars)]
