"""Host-side logic of curvilinear and multi-block problems, on the CPU: metric evaluation,
block splitting, the 4-block topology, and the oracle's interface order (a block cut into
pieces advances exactly like the uncut block)."""
import numpy as np

import harness
from opensbli_gb300 import abi, problems
from opensbli_gb300.spec import BlockSpec


def test_metrics_of_a_uniform_grid_are_the_identity():
    spec = BlockSpec(ndim=3, size=(8, 7, 6), scheme=abi.SCHEME_TENO5, delta=(0.1, 0.2, 0.3))
    grids = []
    for d in range(3):
        n = spec.size[d] + 2 * spec.halo + 4
        shp = [1, 1, 1]
        shp[2 - d] = n
        grids.append(np.broadcast_to(((np.arange(n) - 7) * spec.delta[d]).reshape(shp),
                                     tuple(s + 4 for s in spec.shape)).copy())
    met = problems.metrics_central4(spec, grids, extended=True)
    for d in range(3):
        for i in range(3):
            assert np.allclose(met[3 * d + i], 1.0 if d == i else 0.0, atol=1e-12)
    assert np.allclose(met[9], 1.0, atol=1e-12)


def test_curvilinear_wave_metrics_are_periodic():
    spec, q, met = problems.curvilinear_wave_2d(32)
    h = spec.halo
    for k in (0, 1, 3, 4, 9):
        a = met[k]
        assert np.array_equal(a[:, :h], a[:, 32:32 + h])
        assert np.array_equal(a[:h, :], a[32:32 + h, :])


def test_multiblock_topology_is_symmetric():
    blocks = problems.curvilinear_multiblock_3d(sizes={"A": (32, 16, 8), "B": (16, 16, 8), "C": (32, 8, 8),
                                                       "D": (16, 16, 8)})
    specs = [b[0] for b in blocks]
    for ib, s in enumerate(specs):
        for d in range(3):
            for side in range(2):
                if s.bc[d][side] != abi.BC_INTERFACE:
                    continue
                nb, nd, nside, flip = s.iface[d][side]
                assert nd == d and flip == 0 and nside == 1 - side
                other = specs[nb]
                assert other.bc[d][nside] == abi.BC_INTERFACE
                assert other.iface[d][nside][0] == ib
                for e in range(3):
                    if e != d:
                        assert other.size[e] == s.size[e]
    # the mesh is continuous across every interface: the metric halo of a block equals the
    # neighbour's metric next to the shared face (D_00 and det J checked)
    for ib, (s, _, met) in enumerate(blocks):
        for d in range(3):
            for side in range(2):
                if s.bc[d][side] != abi.BC_INTERFACE:
                    continue
                nb = s.iface[d][side][0]
                ns, _, nmet = blocks[nb]
                ax = 2 - d
                h = s.halo
                for k in (0, 9):
                    mine = np.take(met[k], range(0, h) if side == 0 else range(h + s.size[d], 2 * h + s.size[d]), axis=ax)
                    src = range(ns.size[d], ns.size[d] + h) if side == 0 else range(h, 2 * h)
                    theirs = np.take(nmet[k], src, axis=ax)
                    core = tuple(slice(h, h + s.size[2 - a]) if a != ax else slice(None) for a in range(3))
                    assert np.allclose(mine[core], theirs[core], rtol=0, atol=1e-12), (ib, d, side, k)


def test_oracle_split_block_equals_single_block(oracle_lib):
    rng = np.random.default_rng(3)
    spec, q = problems.tgv(minf=1.25, scheme=abi.SCHEME_TENO5, averaging=abi.AVG_ROE,
                           viscous=abi.VISC_SUTHERLAND, sizes=(20, 12, 12))
    q = [a * (1.0 + 1e-3 * rng.standard_normal(a.shape)) for a in q]
    one = harness.OracleBlocks([(spec, q)])
    parts = problems.split_block(spec, q, [8, 14], d=0)
    many = harness.OracleBlocks(parts)
    A, B = problems.RK3_LS_A, problems.RK3_LS_B
    one.step(abi.RK_LOW_STORAGE, A, B, 1e-3, 2)
    many.step(abi.RK_LOW_STORAGE, A, B, 1e-3, 2)
    sl = spec.interior()
    edges = [0, 8, 14, 20]
    for b, (ps, _) in enumerate(parts):
        for v in range(spec.nvars):
            assert np.array_equal(many.q[b][v][ps.interior()], one.q[0][v][sl][:, :, edges[b]:edges[b + 1]])
