"""Failure detection through the C ABI without faulting the GPU: non-finite values made on the
host are reported by osb_sync as OSB_ENAN (and counted by the NaN reduction) while the context
stays usable, and osb_sync returns OSB_ETIMEDOUT instead of blocking while work is in flight."""
import math

import numpy as np
import pytest

from opensbli_gb300 import abi, problems

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_nan_in_state_is_reported_and_context_recovers(built_lib, precision):
    from opensbli_gb300.solver import Solver
    spec, q = problems.kh(32)
    bad = [a.copy() for a in q]
    h = spec.halo
    bad[0][h + 7, h + 9] = math.nan
    s = Solver([(spec, bad)], precision=precision, rk="ls3")
    s.set_schedule(mode=abi.SCHED_PER_BLOCK)
    s.apply_bc()
    s.step(2e-4, 1)
    with pytest.raises(abi.OSBError) as e:
        s.sync()
    assert "non-finite" in str(e.value)
    assert s.reduce(abi.RED_NAN_COUNT) > 0
    # the same context continues once the caller restores a finite state
    s.q[0].copy_(s.torch.from_numpy(np.stack(q)))
    s.rk[0].zero_()
    s.apply_bc()
    s.step(2e-4, 2)
    s.sync()
    assert s.reduce(abi.RED_NAN_COUNT) == 0
    s.close()


def test_sync_times_out_while_work_is_in_flight(built_lib):
    from opensbli_gb300.solver import Solver
    spec, q = problems.tgv(96, minf=1.25, scheme=abi.SCHEME_TENO5, averaging=abi.AVG_ROE)
    s = Solver([(spec, q)], precision="fp64", rk="ls3")
    s.apply_bc()
    s.step(1e-3, 20)  # tens of milliseconds of queued work
    rc = s.lib.osb_sync(s.ctx, 0)
    assert rc == abi.OSB_ETIMEDOUT, rc
    assert "not idle" in abi.last_error(s.lib)
    s.sync(600000)  # the work completes normally afterwards
    s.close()
