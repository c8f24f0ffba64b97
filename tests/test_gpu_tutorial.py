"""magex's Python-API tutorial (docs/tutorials/07_python_api.md:18-31) through this package:
write_model -> load_results -> supercell -> LLGSolver.run -> topological charge -> Monte Carlo sweeps,
against the same script run by the reference (rows, snapshots, final spins and Q)."""
import numpy as np
import pytest


def _tutorial_system(path):
    from magex_gb300 import Supercell, load_results, write_model
    write_model(str(path), lattice="triangular", J=[2.0], D=1.0, moment=3.0)
    return Supercell(load_results(str(path)), supercell=(48, 48, 1), pbc=(True, True, False), field=(0, 0, 2.0))


def test_tutorial_trajectory_on_the_oracle(golden, tmp_path):
    from oracle import OracleLLG
    s = _tutorial_system(tmp_path / "tri.json")
    ora = OracleLLG(s, 0.5, 2e-3, 0.0)
    e = s.init_spins("random", seed=1)
    for _ in range(20000):
        ora.step_inplace(e)
    assert np.abs(e - golden["tutorial/e"]).max() < 1e-11


@pytest.mark.gpu
def test_tutorial_script(cuda, golden, tmp_path):
    from magex_gb300 import LLGSolver, MetropolisMC, texture
    s = _tutorial_system(tmp_path / "tri.json")
    e = s.init_spins("random", seed=1)
    llg = LLGSolver(s, alpha=0.5, dt=2e-3, temperature=0.0)
    e, table, snaps = llg.run(e, steps=20000, output_every=200, snapshots=10)
    ref = golden["tutorial/table"]
    assert table.shape == ref.shape
    assert np.abs(table - ref).max() < 1e-9
    assert np.abs(e - golden["tutorial/e"]).max() < 1e-9
    assert np.allclose([t for t, _ in snaps], golden["tutorial/snap_t"], rtol=0, atol=1e-12)
    assert np.abs(snaps[5][1] - golden["tutorial/snap5"]).max() < 1e-9
    Q = texture.topological_charge(s, e)
    assert abs(Q - float(golden["tutorial/Q"])) < 1e-9
    mc = MetropolisMC(s, temperature=20.0, seed=3)
    for _ in range(1000):
        e = mc.sweep(e)
    assert np.abs(np.linalg.norm(e, axis=1) - 1).max() < 1e-12
