"""C-ABI checks that need no GPU: the library loads, exports every entry point the header
declares, and the ctypes descriptor layout matches the C struct."""
import ctypes
import os
import re

from opensbli_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    txt = open(os.path.join(ROOT, "include", "osb_gb300.h")).read()
    return sorted(set(re.findall(r"^int (osb_\w+)\(", txt, re.M)))


def test_header_and_binding_agree():
    assert header_functions() == sorted(abi.EXPORTED)


def test_library_exports_every_symbol(built_lib):
    lib = abi.load_library()
    for name in header_functions():
        assert hasattr(lib, name), name


def test_descriptor_layout(built_lib):
    lib = abi.load_library()
    out = (ctypes.c_longlong * 20)()
    assert lib.osb_desc_layout(out, 20) == 0
    assert list(out) == abi.layout_signature()


def test_version_and_errors(built_lib):
    lib = abi.load_library()
    assert lib.osb_version() == 100
    assert lib.osb_desc_layout(None, 0) == abi.OSB_EINVAL
    assert "20 slots" in abi.last_error(lib)


def test_new_entry_points_reject_bad_arguments_without_a_gpu(built_lib):
    """osb_metrics and osb_step_requests validate their arguments before touching the device."""
    lib = abi.load_library()
    vp = ctypes.c_void_p
    assert lib.osb_metrics(None, None, None, 0, None) == abi.OSB_EINVAL
    from opensbli_gb300 import problems
    from opensbli_gb300.spec import BlockSpec
    spec = BlockSpec(ndim=1, size=(16,), delta=(0.1,), scheme=abi.SCHEME_WENO5_JS)
    d = abi.make_desc(spec, [0] * 5, [0] * 5)
    xs = (vp * 3)(0, 0, 0)
    ms = (vp * 10)(*([0] * 10))
    assert lib.osb_metrics(ctypes.byref(d), xs, ms, abi.METRIC_EDGE, None) == abi.OSB_EINVAL
    assert "2D and 3D" in abi.last_error(lib)
    spec, _, _ = problems.curvilinear_wave_2d(16)
    d = abi.make_desc(spec, [0] * 5, [0] * 5)
    assert lib.osb_metrics(ctypes.byref(d), xs, ms, 7, None) == abi.OSB_EINVAL
    assert "fill" in abi.last_error(lib)
    assert lib.osb_step_requests(None, 1, None, None, 1e-3, 1) == abi.OSB_EINVAL


def test_hllc_descriptor_outside_the_gpu_flux_refused(built_lib):
    """The GPU HLLC-LM flux covers Cartesian 2D / 3D blocks with the fifth-order WENO / TENO
    reconstructions; any other combination (here TENO6) is refused loudly, before any device
    work, instead of running the LLF flux in its place."""
    from opensbli_gb300 import problems
    lib = abi.load_library()
    spec, _ = problems.shock_reflection(40, 20, flux_type=abi.FLUX_HLLC_LM)
    spec.scheme = abi.SCHEME_TENO6
    d = abi.make_desc(spec, [1] * 4, [1] * 4, None, {(0, 0): 1, (1, 1): 1})
    assert lib.osb_stage_noalloc(ctypes.byref(d), abi.RK_LOW_STORAGE, 0.0, 0.5, 0.1, None) == abi.OSB_EINVAL
    assert "HLLC" in abi.last_error(lib)


def test_pressure_outlet_without_back_pressure_refused(built_lib):
    """A pressure-outlet face needs its back pressure (osb_block_desc.back_pressure); a face left
    at zero is refused before any device work."""
    from opensbli_gb300 import problems
    lib = abi.load_library()
    spec, _ = problems.shock_reflection(40, 20, back_pressure=0.2)
    d = abi.make_desc(spec, [1] * 4, [1] * 4, None, {(0, 0): 1, (1, 1): 1})
    assert d.back_pressure[0][1] == 0.2
    d.back_pressure[0][1] = 0.0
    assert lib.osb_stage_noalloc(ctypes.byref(d), abi.RK_LOW_STORAGE, 0.0, 0.5, 0.1, None) == abi.OSB_EINVAL
    assert "back pressure" in abi.last_error(lib)


def test_ystretch_metrics_host_function(built_lib):
    """osb_ystretch_metrics (host work, no GPU): a uniform line gives D11 = 1 / x' and SD111 = 0
    to rounding; short, non-monotone and wall-less lines are refused with OSB_EINVAL."""
    import numpy as np
    import pytest
    n, d = 17, 1.0 / 16.0
    x = -1.0 + 2.0 * np.arange(n) / (n - 1)  # x' = 2 on xi in [0, 1]
    d11, sd = abi.ystretch_metrics(x, d)
    assert np.max(np.abs(d11 - 0.5)) < 1e-13 and np.max(np.abs(sd)) < 1e-11
    with pytest.raises(abi.OSBError):
        abi.ystretch_metrics(x[:10], d)  # fewer than 12 rows
    bad = x.copy()
    bad[5] = bad[4]
    bad[6] = bad[4]
    bad[7] = bad[4]
    bad[3] = bad[4]
    with pytest.raises(abi.OSBError):
        abi.ystretch_metrics(bad, d)  # a flat stretch: x' = 0 somewhere
    with pytest.raises(abi.OSBError):
        abi.ystretch_metrics(x, d, wall_lo=False)  # no rule for the rows next to a free end
