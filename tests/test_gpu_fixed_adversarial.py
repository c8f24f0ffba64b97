"""The exact fixed-point exchange sum (precision="fp64_fixed") on models built to break it.

Fixtures: tests/golden/adversarial.npz (make_golden.py --adversarial), magex's own T = 0 Heun
trajectories of (a) a simple-cubic model whose couplings span eight decades in one stencil (100,
1e-3 and 1e-6 meV shells, DMI, a 1e-2 meV anisotropic part), a near-zero single-ion term (1e-9 meV)
and a 100 T field, and (b) a two-site bcc model with four per-shell full tensors (20, 10, -1 and
1e-6 meV), K = 1e-10 meV and the same field.  The per-sublattice scale 2^sigma of the fixed-point
sum is set by the sum of all coupling magnitudes (the 100 meV shell), so the 1e-6 meV couplings are
held with 2^-57 of that scale; the 100 T Zeeman field is added in FP64 outside the sum.  Both the
all-FP64 step and the fixed-point form must follow the reference to 1e-12 per step and 1e-9 after
1000 steps (the bars of the plain FP64 path), and give its energy and effective field.
"""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def adv():
    return np.load(os.path.join(HERE, "golden", "adversarial.npz"))


def _system(meta):
    from magex_gb300.lattice import Supercell
    from magex_gb300.spinmodel import load_results
    return Supercell(load_results(meta["model"], jtol=meta["jtol"]), tuple(meta["L"]), (True, True, True), tuple(meta["B"]))


@pytest.mark.parametrize("precision", ["fp64", "fp64_fixed"])
@pytest.mark.parametrize("tag", ["sc_decades", "bcc2_decades"])
def test_adversarial_trajectory_matches_reference(cuda, adv, tag, precision):
    from magex_gb300.llg import GB300LLG
    meta = json.loads(str(adv["meta"]))[tag]
    sc = _system(meta)
    sol = GB300LLG(sc, meta["alpha"], meta["dt"], 0.0, 1, precision=precision)
    lat = sol.model.to_lattice(adv[f"{tag}/e0"])
    done = 0
    for n in meta["keep"]:
        sol.run_lattice(lat, n - done)
        done = n
        got = sol.model.from_lattice(lat).cpu().numpy()
        err = float(np.abs(got - adv[f"{tag}/e{n}"]).max())
        assert err <= 1e-12 * n, (tag, precision, n, err)
    E = float(adv[f"{tag}/energy"])
    e_end = sol.model.from_lattice(lat).cpu().numpy()
    assert abs(sol.energy(e_end) - E) <= 1e-12 * abs(E)
    B = sol.model.from_lattice(sol.model.effective_field(lat)).cpu().numpy()
    Bref = adv[f"{tag}/field"]
    assert np.abs(B - Bref).max() <= 1e-9 * np.abs(Bref).max()


def test_fixed_point_scale_resolves_the_smallest_shell(cuda, adv):
    """The 1e-6 meV shell is not lost to the 100 meV scale: doubling it changes one step by ~2e-9
    (its field is ~1.4e-4 T), and the fixed-point form sees the same change as the all-FP64 form to
    FP64 rounding; from the same spins the two forms differ by FP64 rounding only."""
    from magex_gb300.lattice import Supercell
    from magex_gb300.llg import GB300LLG
    from magex_gb300.spinmodel import load_results, make_model
    meta = json.loads(str(adv["meta"]))["sc_decades"]
    e0 = adv["sc_decades/e0"]
    steps = {}
    for j3 in (1e-6, 2e-6):
        model = make_model("sc", J=[100.0, 1e-3, j3], D=5.0, Jani=[[1e-2, 0, 0], [0, -2e-2, 0], [0, 0, 1e-2]],
                           K=1e-9, moment=2.0)
        sc = Supercell(load_results(model, jtol=meta["jtol"]), tuple(meta["L"]), (True, True, True), tuple(meta["B"]))
        for prec in ("fp64", "fp64_fixed"):
            steps[j3, prec] = GB300LLG(sc, meta["alpha"], meta["dt"], 0.0, 1, precision=prec).step(e0)
    assert np.abs(steps[1e-6, "fp64"] - steps[1e-6, "fp64_fixed"]).max() <= 1e-15
    d64 = steps[2e-6, "fp64"] - steps[1e-6, "fp64"]
    dfx = steps[2e-6, "fp64_fixed"] - steps[1e-6, "fp64_fixed"]
    assert np.abs(d64).max() > 1e-9
    assert np.abs(dfx - d64).max() <= 2e-15
