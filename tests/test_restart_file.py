"""Restart files on the host (no GPU): the datasets, OPS attributes and constants the reference
restarts from (state of every time-advance array, iter, simulation_time) round-trip exactly."""
import json

import numpy as np
import pytest

from opensbli_gb300 import problems, restart


def test_restart_file_round_trip(tmp_path):
    rng = np.random.default_rng(0)
    s1, q1 = problems.sod(50)
    s2, q2 = problems.kh(sizes=(12, 10))
    regs = [[rng.standard_normal(s.shape) for _ in range(s.nvars)] for s in (s1, s2)]
    path = str(tmp_path / "r.npz")
    restart.write(path, [s1, s2], [q1, q2], regs, 17, 0.25)
    data = restart.read(path)
    assert data["iter"] == 17 and data["simulation_time"] == 0.25
    restart.check_compatible([s1, s2], data)
    for b, (q, r) in enumerate(((q1, regs[0]), (q2, regs[1]))):
        blk = data["blocks"][b]
        assert all(np.array_equal(x, y) for x, y in zip(blk["state"], q))
        assert all(np.array_equal(x, y) for x, y in zip(blk["register"], r))
    with np.load(path) as f:
        meta = json.loads(str(f["meta"]))
        assert "opensbliblock01/rhou1_B1" in f.files and "opensbliblock00/rhoE_RKold_B0" in f.files
    att = meta["blocks"][1]["datasets"]["rho_B1"]
    assert att["d_m"] == [-5, -5] and att["d_p"] == [5, 5] and att["size"] == [12, 10] and att["block_index"] == 1


def test_restart_file_checks(tmp_path):
    s, q = problems.sod(50)
    path = str(tmp_path / "r.npz")
    restart.write(path, [s], [q], [q], 0, 0.0)
    other, _ = problems.sod(60)
    with pytest.raises(ValueError):
        restart.check_compatible([other], restart.read(path))
    with pytest.raises(ValueError):
        restart.write(path, [s], [q[:2]], [q], 0, 0.0)
    np.savez(str(tmp_path / "x.npz"), meta=np.array(json.dumps({"format": "something else"})))
    with pytest.raises(ValueError):
        restart.read(str(tmp_path / "x.npz"))
