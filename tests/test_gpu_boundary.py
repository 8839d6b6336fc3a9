"""Boundary kernels on the GPU against the oracle and against the periodic definition, halos
included: a block whose faces are all periodic gets its whole halo shell in one launch, which
must leave exactly what the direction-by-direction exchange of the reference (ExchangeSelf,
periodic.py:53-71, x then y then z with corners) leaves."""
import numpy as np
import pytest

import harness
from opensbli_gb300 import abi, problems

pytestmark = pytest.mark.gpu


def _scramble(q, seed):
    """Random values everywhere, halos included, so stale halos cannot pass by accident."""
    rng = np.random.default_rng(seed)
    return [1.0 + rng.random(a.shape) for a in q]


def _wrapped(a, spec, depth):
    """The interior of `a` wrapped onto the box [-depth, N + depth) of every used direction."""
    h = spec.halo
    idx = []
    for ax in range(a.ndim):
        d = spec.ndim - 1 - ax  # arrays are (z, y, x)
        n = spec.size[d]
        c = np.arange(-depth, n + depth)
        idx.append(h + np.mod(c, n))
    return a[np.ix_(*idx)]


def _box(a, spec, depth):
    h = spec.halo
    return a[tuple(slice(h - depth, h + spec.size[spec.ndim - 1 - ax] + depth) for ax in range(a.ndim))]


@pytest.mark.parametrize("case", ["3d", "2d", "1d"])
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_periodic_shell_matches_exchange_and_wrap(built_lib, case, precision):
    from opensbli_gb300.solver import Solver
    if case == "3d":
        spec, q = problems.tgv(sizes=(11, 7, 6), scheme=abi.SCHEME_TENO5, averaging=abi.AVG_ROE)
    elif case == "2d":
        spec, q = problems.kh(sizes=(9, 6))
    else:
        spec, q = problems.sod(13, bc=(abi.BC_PERIODIC, abi.BC_PERIODIC))
    depth = spec.bc_depth[0][0]
    q = _scramble(q, 3)
    s = Solver([(spec, q)], precision=precision, rk="ls3")
    s.apply_bc()
    got = s.state(0)
    s.close()
    ob = harness.OracleBlocks([(spec, q)])
    ob.apply_bc()
    ref = ob.q[0]
    for v in range(spec.nvars):
        assert np.array_equal(got[v], ref[v]), (case, v, "oracle")
        assert np.array_equal(_box(got[v], spec, depth), _wrapped(got[v], spec, depth)), (case, v, "wrap")
