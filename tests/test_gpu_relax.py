"""Damped-LLG relaxation (magex_gb300.minimize) against magex/minimize.py:168-181 run by the reference:
same stopping check, same iteration count, spins and energy to the FP64 bars."""
import numpy as np
import pytest

from helpers import apply_structure_subset

CASES = ("tri", "sc_pinned", "max_iter")


def _system(golden_models, tag):
    from magex_gb300.lattice import Supercell
    from magex_gb300.spinmodel import load_results
    c = golden_models["relax"][tag]
    sc = Supercell(load_results(golden_models[c["model"]]["model"]), tuple(c["L"]), tuple(c["pbc"]), tuple(c["B"]))
    if c["structure"]:
        apply_structure_subset(sc, c["structure"])
    return sc, c


@pytest.mark.gpu
@pytest.mark.parametrize("tag", CASES)
def test_llg_relaxation_matches_reference(cuda, golden, golden_models, tag):
    from magex_gb300.minimize import minimize
    sc, c = _system(golden_models, tag)
    e, info = minimize(sc, golden[f"relax/{tag}/e0"], "llg", tol=c["tol"], max_iter=c["max_iter"])
    assert info["iterations"] == int(golden[f"relax/{tag}/iterations"])
    assert np.abs(e - golden[f"relax/{tag}/e"]).max() < 1e-9
    E = float(golden[f"relax/{tag}/energy"])
    assert abs(info["energy"] - E) <= 1e-10 * abs(E)


@pytest.mark.parametrize("tag", CASES)
def test_oracle_relaxation_matches_reference(golden, golden_models, tag):
    """The loop of magex/minimize.py:168-181 over the oracle's step pins the stopping rule and the
    iteration count that the device relaxation must reproduce."""
    from oracle import MU_B, OracleLLG
    sc, c = _system(golden_models, tag)
    ora = OracleLLG(sc, 1.0, 2e-3, 0.0, precession=False)
    e = np.ascontiguousarray(golden[f"relax/{tag}/e0"], np.float64).copy()
    n = c["max_iter"] or 100000
    for it in range(n):
        if it % 50 == 0 and ora.observables(e)[7] * MU_B * float(np.max(sc.mu)) < c["tol"]:
            break
        ora.step_inplace(e)
    assert it == int(golden[f"relax/{tag}/iterations"])
    assert np.abs(e - golden[f"relax/{tag}/e"]).max() < 1e-9


def test_host_methods_are_refused(golden_models):
    from magex_gb300.minimize import minimize
    sc, _ = _system(golden_models, "tri")
    e = sc.init_spins("random", seed=1)
    for m in ("lbfgs", "ncg", "vp"):
        with pytest.raises(NotImplementedError):
            minimize(sc, e, m)
    with pytest.raises(ValueError):
        minimize(sc, e, "newton")
