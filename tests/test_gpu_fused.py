"""The FP32-residual stage applies the RK update inside its last residual kernel (central
kernel, or the last sweep of an Euler block) and ping-pongs the FP32 state between two buffers.
Checked here against the unfused pieces through the C ABI: the residual hook (osb_residual,
the same kernels without the update) followed by the RK update in numpy (FP64), per block, for
every kind of last kernel.  The update takes dt * residual rounded once to FP32 (at most 2^-24 of the increment, below
the residual's own FP32 error) and forms the register and the state with FP64 FMAs, so the
register agrees to 2^-24 of dt * residual and the state to that times |B|, plus FP64 rounding."""
import numpy as np
import pytest

from opensbli_gb300 import abi, problems

pytestmark = pytest.mark.gpu

A, B = problems.RK3_LS_A, problems.RK3_LS_B


def _cases():
    rng = np.random.default_rng(4)

    def pert(q):
        return [a * (1.0 + 1e-3 * rng.standard_normal(a.shape)) for a in q]
    out = {}
    spec, q = problems.tgv(16, minf=1.25, scheme=abi.SCHEME_TENO5, averaging=abi.AVG_ROE)
    out["tgv_teno5_viscous"] = ([(spec, q)], 1e-3)            # last kernel: central (viscous)
    spec, q = problems.tgv(16, minf=0.1, scheme=abi.SCHEME_CENTRAL4)
    out["tgv_central4"] = ([(spec, q)], 3.385e-3)              # only kernel: central (conv + visc)
    spec, q = problems.tgv(16, minf=1.25, scheme=abi.SCHEME_TENO5, averaging=abi.AVG_ROE, viscous=abi.VISC_NONE)
    out["tgv_teno5_euler"] = ([(spec, pert(q))], 1e-3)         # last kernel: z sweep
    spec, q = problems.kh(32)
    out["kh_euler_2d"] = ([(spec, pert(q))], 2e-4)             # last kernel: y sweep
    out["curv_multiblock"] = (problems.curvilinear_multiblock_3d(
        sizes={"A": (32, 16, 8), "B": (16, 16, 8), "C": (32, 8, 8), "D": (16, 16, 8)}, seed=3), 5e-3)
    spec, q = problems.sod(200)
    out["sod_1d"] = ([(spec, q)], 2e-4)                        # 1D: separate RK kernel
    return out


CASES = _cases()


@pytest.mark.parametrize("name", sorted(CASES))
def test_fused_stage_matches_residual_plus_update(built_lib, name):
    from opensbli_gb300.solver import Solver
    blocks, dt = CASES[name]
    s = Solver(blocks, precision="fp32", rk="ls3")
    s.set_schedule(mode=abi.SCHED_PER_BLOCK)
    s.apply_bc()
    s.stage(0, dt)  # leaves a non-trivial RK register for the second stage
    q0 = [s.state(i) for i in range(len(blocks))]
    r0 = [s.rk_register(i) for i in range(len(blocks))]
    R = [s.residual(i) for i in range(len(blocks))]
    s.stage(1, dt)
    q1 = [s.state(i) for i in range(len(blocks))]
    r1 = [s.rk_register(i) for i in range(len(blocks))]
    s.close()
    for i, blk in enumerate(blocks):
        spec = blk[0]
        sl = spec.interior()
        for v in range(spec.nvars):
            o = A[1] * r0[i][v][sl] + dt * R[i][v][sl]
            qn = B[1] * o + q0[i][v][sl]
            # dt * residual enters rounded once to FP32: |error| <= 2^-24 |dt R| per point; the
            # FMAs add FP64 rounding on the scale of the terms they sum
            inc = np.abs(dt * R[i][v][sl])
            scale_o = max(float(np.max(np.abs(o))), float(np.max(inc)),
                          float(np.max(np.abs(A[1] * r0[i][v][sl]))), 1e-300)
            scale_q = max(float(np.max(np.abs(qn))), 1e-300)
            bound_o = 2.0 ** -24 * inc + 1e-14 * scale_o
            bound_q = abs(B[1]) * 2.0 ** -24 * inc + 1e-14 * scale_q
            assert np.all(np.abs(r1[i][v][sl] - o) <= bound_o), (name, i, v, "register")
            assert np.all(np.abs(q1[i][v][sl] - qn) <= bound_q), (name, i, v, "state")


@pytest.mark.parametrize("variant", [1, 2, 3, 4, 5])
def test_x_sweep_variants_are_bit_identical(built_lib, variant):
    """The x-sweep segment length (osb_set_variant) changes only the tiling: same states.
    70^3: 4 900 rows leave a partial last warp, segments of 64 and 32 leave ragged ends."""
    from opensbli_gb300.solver import Solver
    spec, q = problems.tgv(70, minf=1.25, scheme=abi.SCHEME_TENO5, averaging=abi.AVG_ROE)
    out = []
    for var in (0, variant):
        s = Solver([(spec, q)], precision="fp32", rk="ls3")
        s.set_variant(var)
        s.apply_bc()
        s.step(1e-3, 2)
        out.append(s.state(0))
        s.close()
    for v in range(spec.nvars):
        assert np.array_equal(out[0][v], out[1][v]), v


def _bulk_cases():
    out = {}
    spec, q = problems.tgv(16, minf=1.25, scheme=abi.SCHEME_TENO5, averaging=abi.AVG_ROE,
                           sizes=(37, 21, 19))  # x beyond one 32-wide tile, ragged y tiles, odd z
    out["teno5_viscous_ragged"] = ([(spec, q)], 1e-3)
    spec, q = problems.tgv(16, minf=0.1, scheme=abi.SCHEME_CENTRAL4, sizes=(64, 12, 40))
    out["central4_feiereisen"] = ([(spec, q)], 3.385e-3)
    spec, q = problems.tgv_filtered(16, sizes=(40, 36, 24))  # KGP form (eleven ring fields)
    spec.filter = abi.FILTER_NONE
    out["central4_kgp"] = ([(spec, q)], 1e-3)
    spec, q = problems.tgv_filtered(16, sizes=(64, 608, 6))  # 4-row tiles (many 32 x 4 columns)
    spec.filter = abi.FILTER_NONE
    out["central4_kgp_4rows"] = ([(spec, q)], 1e-3)
    return out


BULK_CASES = _bulk_cases()


@pytest.mark.parametrize("name", sorted(BULK_CASES))
def test_central_bulk_staging_is_bit_identical(built_lib, name):
    """The central kernel's planes staged by bulk copies (cp.async.bulk + mbarrier) and by
    per-thread register loads give bit-identical states and RK registers over two steps."""
    from opensbli_gb300.solver import Solver
    blocks, dt = BULK_CASES[name]
    got = []
    for bulk in (0, 1):
        s = Solver(blocks, precision="fp32", rk="ls3", graphs=bool(bulk))
        s.set_schedule(mode=abi.SCHED_PER_BLOCK, fuse_update=1)
        s.set_central_staging(bulk)
        s.apply_bc()
        s.step(dt, 2)
        s.sync()
        got.append(([s.state(i) for i in range(len(blocks))], [s.rk_register(i) for i in range(len(blocks))]))
        s.close()
    for i, blk in enumerate(blocks):
        sl = blk[0].interior()
        for v in range(blk[0].nvars):
            assert np.array_equal(got[0][0][i][v], got[1][0][i][v]), (name, i, v, "state")
            assert np.array_equal(got[0][1][i][v][sl], got[1][1][i][v][sl]), (name, i, v, "register")
