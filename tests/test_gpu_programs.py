"""FMR ring-down (magex_gb300.programs.fmr) against magex/programs.py:124-150 run by the reference."""
import numpy as np
import pytest

CASES = ("tri_heun", "sc_depondt")


def _system(golden_models, tag):
    from magex_gb300.lattice import Supercell
    from magex_gb300.spinmodel import load_results
    c = golden_models["fmr"][tag]
    return Supercell(load_results(golden_models[c["model"]]["model"]), tuple(c["L"]), tuple(c["pbc"]),
                     tuple(c["B"])), c["kw"]


@pytest.mark.parametrize("tag", CASES)
def test_peak_refinement_matches_reference(golden, tag):
    from magex_gb300.programs import _peak_frequency
    f, F = golden[f"fmr/{tag}/f"], golden[f"fmr/{tag}/F"]
    assert abs(_peak_frequency(f, F) - float(golden[f"fmr/{tag}/fpk"])) < 1e-9


@pytest.mark.parametrize("tag", CASES)
def test_oracle_ring_down_matches_reference(golden, golden_models, tag):
    """The pulse (on while a stage's time is below 5 dt) and the sampling (after every step n with
    n % every == 0), restated over the oracle's two stages, reproduce the reference's table."""
    from oracle import OracleLLG
    sc, kw = _system(golden_models, tag)
    dt, every, steps = kw["dt"], kw["every"], kw["steps"]
    p = np.asarray(kw.get("direction", (1, 0, 0)), float)
    p = p / np.linalg.norm(p)
    ora = OracleLLG(sc, kw["alpha"], dt, 0.0, integrator=kw.get("integrator", "heun"))
    B0 = np.asarray(sc.B, float).copy()
    e = np.ascontiguousarray(golden[f"fmr/{tag}/e"], np.float64).copy()
    t, rows = 0.0, []
    for n in range(steps):
        for stage, ts in ((0, t), (1, t + dt)):
            sc.B = B0 + (kw["B_pulse"] * p if ts < 5 * dt else 0.0)
            ora.stage(e, None, stage)
        sc.B = B0
        t += dt
        if n % every == 0:
            rows.append([t, *e.mean(0)])
    ref = golden[f"fmr/{tag}/table"]
    assert np.abs(np.array(rows) - ref).max() < 1e-9


@pytest.mark.gpu
@pytest.mark.parametrize("tag", CASES)
def test_fmr_matches_reference(cuda, golden, golden_models, tag):
    from magex_gb300.programs import fmr
    sc, kw = _system(golden_models, tag)
    (f, F), fpk, table = fmr(sc, golden[f"fmr/{tag}/e"], **kw)
    ref = golden[f"fmr/{tag}/table"]
    assert table.shape == ref.shape
    assert np.abs(table - ref).max() < 1e-9
    assert np.array_equal(f, golden[f"fmr/{tag}/f"])
    Fr = golden[f"fmr/{tag}/F"]
    assert np.abs(F - Fr).max() <= 1e-6 * Fr.max()
    assert abs(fpk - float(golden[f"fmr/{tag}/fpk"])) < 1e-6
