"""On-GPU metric generation (osb_metrics) against the host restatement of the generated metric
kernels (problems.metrics_central4): bit for bit in 2D (the same operator order, no
contraction), to rounding in 3D (cofactor inverse on the GPU, LAPACK on the host)."""
import math

import numpy as np
import pytest

from opensbli_gb300 import abi, problems
from opensbli_gb300.spec import BlockSpec

pytestmark = pytest.mark.gpu


def _np(t):
    return None if t is None else t.cpu().numpy()


@pytest.mark.parametrize("fill", [abi.METRIC_PERIODIC, abi.METRIC_EDGE])
def test_metrics_2d_bit_exact(built_lib, fill):
    from opensbli_gb300.solver import device_metrics
    spec, _, _ = problems.curvilinear_wave_2d(24)
    x = problems.wave_2d_coords(spec)
    want = problems.metrics_central4(spec, list(x), periodic_from_interior=fill == abi.METRIC_PERIODIC)
    got = device_metrics(spec, x, fill)
    for k in (0, 1, 3, 4, 9):
        assert np.array_equal(_np(got[k]), want[k]), k
    assert got[2] is None and got[5] is None


def _mesh_3d(spec, amp=0.05):
    """A periodic wavy 3D mesh at every allocated point (x = xi + amp sin(2 pi eta / L_eta) ...)."""
    g = [spec.grid_index(d).astype(np.float64) * spec.delta[d] for d in range(3)]
    L = [spec.size[d] * spec.delta[d] for d in range(3)]
    s = [np.sin(2 * math.pi * g[d] / L[d]) for d in range(3)]
    x = g[0] + amp * s[1] * s[2]
    y = g[1] + amp * s[0] * s[2]
    z = g[2] + amp * s[0] * s[1]
    return [np.broadcast_to(a, spec.shape).copy() for a in (x, y, z)]


@pytest.mark.parametrize("fill", [abi.METRIC_PERIODIC, abi.METRIC_EDGE])
def test_metrics_3d(built_lib, fill):
    from opensbli_gb300.solver import device_metrics
    spec = BlockSpec(ndim=3, size=(14, 11, 9), delta=(1.0 / 14, 1.0 / 11, 1.0 / 9), scheme=abi.SCHEME_TENO5)
    x = _mesh_3d(spec)
    want = problems.metrics_central4(spec, x, periodic_from_interior=fill == abi.METRIC_PERIODIC)
    got = device_metrics(spec, x, fill)
    for k in range(10):
        g, w = _np(got[k]), want[k]
        assert np.max(np.abs(g - w)) <= 1e-13 * max(1.0, np.max(np.abs(w))), k


def test_metrics_rejects_bad_arguments(built_lib):
    from opensbli_gb300.solver import device_metrics
    spec = BlockSpec(ndim=3, size=(4, 11, 9), delta=(0.25, 1.0 / 11, 1.0 / 9), scheme=abi.SCHEME_TENO5)
    with pytest.raises(abi.OSBError):  # fewer points than the periodic halo
        device_metrics(spec, _mesh_3d(spec), abi.METRIC_PERIODIC)
    spec = BlockSpec(ndim=1, size=(16,), delta=(0.1,), scheme=abi.SCHEME_WENO5_JS)
    with pytest.raises(abi.OSBError):
        device_metrics(spec, [np.zeros(spec.shape)], abi.METRIC_EDGE)
