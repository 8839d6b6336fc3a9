"""ctypes mirror of ``include/osb_gb300.h`` and loader of the CUDA library.

The structure layout must match the C header field for field; ``tests/test_abi.py`` checks
the size and offsets against the compiled library (``osb_desc_layout``).
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_NAME = "libosb_gb300.so"

OSB_OK = 0
OSB_EINVAL = -1
OSB_ECUDA = -2
OSB_ETIMEDOUT = -3
OSB_ENOTSUP = -4
OSB_ENAN = -5

SCHEME_WENO5_JS = 1
SCHEME_WENO5_Z = 2
SCHEME_TENO5 = 3
SCHEME_TENO6 = 4
SCHEME_CENTRAL4 = 5

AVG_SIMPLE = 0
AVG_ROE = 1

VISC_NONE = 0
VISC_SUTHERLAND = 1
VISC_CONSTANT = 2
VISC_POWER_LAW = 3  # mu = T^visc_power (the TENO channel app)
VISC_SUTHERLAND_RATIO = 4  # mu = T^1.5 (1 + S) / (T + S), S = SuthT / RefT: oracle only

BC_PERIODIC = 0
BC_ZERO_GRAD = 1
BC_INTERFACE = 2
BC_EXTRAP0 = 3
BC_EXTRAP1 = 4
BC_SYMMETRY = 5
BC_DIRICHLET = 6
BC_PRESSURE_OUTLET = 7
BC_ISOTHERMAL_WALL = 8
BC_ADIABATIC_WALL = 9
BC_INLET_PRESSURE_EXTRAP = 10  # oracle only (the GPU path refuses it)
SPLIT_FEIEREISEN = 0
SPLIT_KGP = 1
FILTER_NONE = 0
FILTER_WENO3 = 1
FILTER_TVD = 2

FLUX_LLF = 0
FLUX_HLLC_LM = 1

METRIC_PERIODIC = 0
METRIC_EDGE = 1

PREC_FP64 = 0
PREC_FP32_RESIDUAL = 1

RK_LOW_STORAGE = 0
RK_SBLI3 = 1

RED_KE = 0
RED_ENSTROPHY_DISS = 1
RED_DILATATION_DISS = 2
RED_RHO_SUM = 3
RED_CFL_DT = 4
RED_NAN_COUNT = 5

SCHED_AUTO = -1
SCHED_PER_BLOCK = 0
SCHED_PERSISTENT = 1


class Schedule(ctypes.Structure):
    """osb_schedule: stage schedule and persistent-stage tiling knobs."""
    _fields_ = [("mode", ctypes.c_int32), ("tile_y", ctypes.c_int32), ("ctas_per_sm", ctypes.c_int32),
                ("dynamic", ctypes.c_int32), ("order", ctypes.c_int32), ("fuse_update", ctypes.c_int32)]

    def as_dict(self):
        return {f: int(getattr(self, f)) for f, _ in self._fields_}


SCHEME_NAMES = {"weno5_js": SCHEME_WENO5_JS, "weno5_z": SCHEME_WENO5_Z, "teno5": SCHEME_TENO5, "teno6": SCHEME_TENO6,
                "central4": SCHEME_CENTRAL4}


class Interface(ctypes.Structure):
    _fields_ = [("block", ctypes.c_int32), ("dir", ctypes.c_int32), ("side", ctypes.c_int32),
                ("flip", ctypes.c_int32)]


class BlockDesc(ctypes.Structure):
    _fields_ = [
        ("ndim", ctypes.c_int32),
        ("size", ctypes.c_int32 * 3),
        ("halo", ctypes.c_int32),
        ("scheme", ctypes.c_int32),
        ("averaging", ctypes.c_int32),
        ("viscous", ctypes.c_int32),
        ("bc", (ctypes.c_int32 * 2) * 3),
        ("bc_depth", (ctypes.c_int32 * 2) * 3),
        ("iface", (Interface * 2) * 3),
        ("gama", ctypes.c_double),
        ("Minf", ctypes.c_double),
        ("Re", ctypes.c_double),
        ("Pr", ctypes.c_double),
        ("mu_const", ctypes.c_double),
        ("eps", ctypes.c_double),
        ("teno_ct", ctypes.c_double),
        ("shock_filter_control", ctypes.c_double),
        ("delta", ctypes.c_double * 3),
        ("q", ctypes.c_void_p * 5),
        ("rkold", ctypes.c_void_p * 5),
        ("metric", ctypes.c_void_p * 10),
        ("split_form", ctypes.c_int32),
        ("filter", ctypes.c_int32),
        ("ducros_check", ctypes.c_double),
        ("ducros_select", ctypes.c_double),
        ("tvd_kappa", ctypes.c_double),
        ("dirichlet", (ctypes.c_void_p * 2) * 3),
        ("flux_type", ctypes.c_int32),
        ("back_pressure", (ctypes.c_double * 2) * 3),
        ("wall_temperature", (ctypes.c_double * 2) * 3),
        ("ystretch", ctypes.c_void_p * 2),
        ("visc_power", ctypes.c_double),
        ("forcing", ctypes.c_double * 3),
        ("sutherland_s", ctypes.c_double),
    ]


def layout_signature():
    """(sizeof, offsets...) of BlockDesc, compared with the C side in the tests."""
    offs = [BlockDesc.size.offset, BlockDesc.bc.offset, BlockDesc.iface.offset, BlockDesc.gama.offset,
            BlockDesc.delta.offset, BlockDesc.q.offset, BlockDesc.rkold.offset, BlockDesc.metric.offset,
            BlockDesc.split_form.offset, BlockDesc.ducros_check.offset, BlockDesc.tvd_kappa.offset,
            BlockDesc.dirichlet.offset, BlockDesc.flux_type.offset, BlockDesc.back_pressure.offset,
            BlockDesc.wall_temperature.offset, BlockDesc.ystretch.offset, BlockDesc.visc_power.offset,
            BlockDesc.forcing.offset, BlockDesc.sutherland_s.offset]
    return [ctypes.sizeof(BlockDesc)] + offs


def make_desc(spec, q_ptrs, rk_ptrs, metric_ptrs=None, dirichlet_ptrs=None, ystretch_ptrs=None):
    """Fill a BlockDesc from a BlockSpec (see backend.py) and raw array addresses
    (ystretch_ptrs: the D11 and SD111 rows of a stretched wall-normal grid)."""
    d = BlockDesc()
    d.ndim = spec.ndim
    for i in range(3):
        d.size[i] = spec.size[i] if i < spec.ndim else 1
        d.delta[i] = spec.delta[i] if i < spec.ndim else 1.0
    d.halo = spec.halo
    d.scheme = spec.scheme
    d.averaging = spec.averaging
    d.viscous = spec.viscous
    for i in range(3):
        for s in range(2):
            if i < spec.ndim:
                d.bc[i][s] = spec.bc[i][s]
                d.bc_depth[i][s] = spec.bc_depth[i][s]
                if spec.iface is not None and spec.iface[i][s] is not None:
                    blk, dr, sd, fl = spec.iface[i][s]
                    d.iface[i][s] = Interface(blk, dr, sd, fl)
    d.gama = spec.gama
    d.Minf = spec.Minf
    d.Re = spec.Re
    d.Pr = spec.Pr
    d.mu_const = spec.mu_const
    d.eps = spec.eps
    d.teno_ct = spec.teno_ct
    d.shock_filter_control = spec.shock_filter_control
    d.split_form = spec.split_form
    d.filter = spec.filter
    d.ducros_check = spec.ducros_check
    d.ducros_select = spec.ducros_select
    d.tvd_kappa = spec.tvd_kappa
    d.flux_type = spec.flux_type
    d.visc_power = spec.visc_power
    d.sutherland_s = spec.sutherland_s
    for i, c in enumerate(spec.forcing or (0.0, 0.0, 0.0)):
        d.forcing[i] = c
    for (i, side), bp in (spec.back_pressure or {}).items():
        d.back_pressure[i][side] = bp
    for (i, side), tw in (spec.wall_temperature or {}).items():
        d.wall_temperature[i][side] = tw
    for v, p in enumerate(q_ptrs):
        d.q[v] = p
    for v, p in enumerate(rk_ptrs):
        d.rkold[v] = p
    if metric_ptrs:
        for i, p in enumerate(metric_ptrs):
            d.metric[i] = p
    if dirichlet_ptrs:
        for (i, side), p in dirichlet_ptrs.items():
            d.dirichlet[i][side] = p
    if ystretch_ptrs:
        d.ystretch[0], d.ystretch[1] = ystretch_ptrs
    return d


class OSBError(RuntimeError):
    pass


_lib = None


def lib_path():
    return os.path.join(HERE, LIB_NAME)


def load_library():
    """Load the in-tree CUDA library.  There is no fallback: a missing library is an error."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        raise OSBError("%s is not built; run `python -c 'import __graft_entry__ as g; g.build()'`" % path)
    lib = ctypes.CDLL(path)
    vp = ctypes.c_void_p
    i32 = ctypes.c_int
    lib.osb_version.restype = i32
    lib.osb_last_error.argtypes = [ctypes.c_char_p, ctypes.c_size_t]
    lib.osb_ctx_create.argtypes = [i32, i32, ctypes.POINTER(vp)]
    lib.osb_ctx_destroy.argtypes = [vp]
    lib.osb_block_add.argtypes = [vp, ctypes.POINTER(BlockDesc), ctypes.POINTER(i32)]
    lib.osb_set_rk.argtypes = [vp, i32, i32, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
    lib.osb_step.argtypes = [vp, ctypes.c_double, i32]
    lib.osb_step_requests.argtypes = [vp, i32, ctypes.POINTER(vp), ctypes.POINTER(vp), ctypes.c_double, i32]
    lib.osb_stage.argtypes = [vp, i32, ctypes.c_double]
    lib.osb_apply_bc.argtypes = [vp]
    lib.osb_residual.argtypes = [vp, i32, ctypes.POINTER(vp)]
    lib.osb_reduce.argtypes = [vp, i32, ctypes.POINTER(ctypes.c_double)]
    lib.osb_sync.argtypes = [vp, i32]
    lib.osb_set_graphs.argtypes = [vp, i32]
    lib.osb_set_variant.argtypes = [vp, i32]
    lib.osb_set_central_staging.argtypes = [vp, i32]
    lib.osb_launch_count.argtypes = [vp, ctypes.POINTER(ctypes.c_longlong)]
    lib.osb_get_stream.argtypes = [vp, ctypes.POINTER(vp)]
    lib.osb_desc_layout.argtypes = [ctypes.POINTER(ctypes.c_longlong), i32]
    lib.osb_metrics.argtypes = [ctypes.POINTER(BlockDesc), ctypes.POINTER(vp), ctypes.POINTER(vp), i32, vp]
    dp = ctypes.POINTER(ctypes.c_double)
    lib.osb_ystretch_metrics.argtypes = [i32, ctypes.c_double, dp, i32, i32, dp, dp]
    lib.osb_stage_noalloc.argtypes = [ctypes.POINTER(BlockDesc), i32, ctypes.c_double, ctypes.c_double,
                                      ctypes.c_double, vp]
    lib.osb_set_schedule.argtypes = [vp, ctypes.POINTER(Schedule)]
    lib.osb_get_schedule.argtypes = [vp, ctypes.POINTER(i32), ctypes.POINTER(Schedule)]
    lib.osb_timing.argtypes = [vp, i32]
    lib.osb_timing_report.argtypes = [vp, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_longlong), i32]
    _lib = lib
    return lib


def last_error(lib):
    buf = ctypes.create_string_buffer(1024)
    lib.osb_last_error(buf, 1024)
    return buf.value.decode(errors="replace")


def ystretch_metrics(x1, delta, wall_lo=True, wall_hi=True):
    """(D11, SD111) of a wall-normal grid line x1 (its interior rows) by osb_ystretch_metrics:
    host work of the library, no GPU needed."""
    import numpy as np
    lib = load_library()
    x = np.ascontiguousarray(x1, dtype=np.float64)
    n = x.shape[0]
    d11, sd = np.zeros(n), np.zeros(n)
    dp = ctypes.POINTER(ctypes.c_double)
    check(lib, lib.osb_ystretch_metrics(n, float(delta), x.ctypes.data_as(dp), int(wall_lo), int(wall_hi),
                                        d11.ctypes.data_as(dp), sd.ctypes.data_as(dp)), "osb_ystretch_metrics")
    return d11, sd


def check(lib, rc, what):
    if rc != OSB_OK:
        raise OSBError("%s failed (%d): %s" % (what, rc, last_error(lib)))
    return rc


# Exported symbols the header declares (checked by the CPU tests without a GPU).
EXPORTED = ["osb_version", "osb_last_error", "osb_ctx_create", "osb_ctx_destroy", "osb_block_add",
            "osb_set_rk", "osb_step", "osb_step_requests", "osb_stage", "osb_apply_bc", "osb_residual", "osb_reduce",
            "osb_sync", "osb_set_graphs", "osb_set_variant", "osb_set_central_staging", "osb_launch_count", "osb_get_stream",
            "osb_desc_layout", "osb_timing", "osb_timing_report", "osb_stage_noalloc", "osb_set_schedule",
            "osb_get_schedule", "osb_metrics", "osb_ystretch_metrics"]

NOALLOC_MAX_DOUBLES = 4 * 1024 * 1024

KERNEL_FAMILIES = ["flux_x", "flux_y", "flux_z", "central", "rk_update", "boundary", "reduce", "persistent_stage",
                   "filter"]
