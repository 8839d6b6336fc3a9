"""osb_step_requests: independent runs from pinned host memory with the copies overlapping the
steps give exactly the states of plain osb_step runs from the same inputs."""
import numpy as np
import pytest

from opensbli_gb300 import abi, problems

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_requests_match_plain_steps(built_lib, precision):
    import torch
    from opensbli_gb300.solver import Solver
    spec, q = problems.tgv(20, minf=1.25, scheme=abi.SCHEME_TENO5, averaging=abi.AVG_ROE)
    rng = np.random.default_rng(7)
    inputs = [[a * (1.0 + 1e-3 * r * rng.standard_normal(a.shape)) for a in q] for r in range(4)]
    dt, nsteps = 1e-3, 2
    # plain runs
    want = []
    for st in inputs:
        s = Solver([(spec, st)], precision=precision, rk="ls3")
        s.apply_bc()
        s.step(dt, nsteps)
        want.append(np.stack(s.state(0)))
        s.close()
    # one context, four requests from pinned host buffers
    s = Solver([(spec, q)], precision=precision, rk="ls3")
    host_in = [torch.from_numpy(np.stack(st)).pin_memory() for st in inputs]
    host_out = [torch.empty_like(h).pin_memory() for h in host_in]
    s.step_requests(host_in, host_out, dt, nsteps)
    n0 = s.launches()
    s.step_requests(host_in[:1], host_out[:1], dt, nsteps)  # a repeat of request 0
    assert s.launches() > n0
    sl = spec.interior()
    for r in range(4):
        got = host_out[r].numpy()
        for v in range(5):
            assert np.array_equal(got[v][sl], want[r][v][sl]), (r, v)
    with pytest.raises(ValueError):
        s.step_requests([host_in[0][:1]], [host_out[0]], dt, 1)
    s.close()
