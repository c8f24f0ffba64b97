"""The CPU oracle against trajectories produced by the reference (tests/golden/make_golden.py).

Pins the oracle before it is trusted as the checker of the GPU kernels: every golden trajectory of
the reference's NumPy path (Heun, Depondt, thermal with the reference's own noise stream, open
boundaries, self-image folding, structure edits) is reproduced to round-off.
"""
import numpy as np
import pytest

from helpers import golden_supercell
from oracle import OracleLLG

TRAJ = ["sc16", "sc6_thermal", "bcc2_thermal", "bcc2_T0", "bcc2_shell4", "tri16", "sc_depondt", "tri_depondt_thermal",
        "sc_open", "sc_tiny_fold", "sc_afm", "honeycomb", "sc_structure", "sc_cubic", "tri_cubic_thermal"]


def _oracle(golden_models, tag, csr="blocks"):
    sc, meta = golden_supercell(golden_models, tag)
    ora = OracleLLG(sc, meta["alpha"], meta["dt"], meta["T"], meta["seed"], integrator=meta["integrator"], csr=csr)
    return sc, meta, ora


@pytest.mark.parametrize("tag", TRAJ)
def test_oracle_trajectory(golden, golden_models, tag):
    sc, meta, ora = _oracle(golden_models, tag)
    e = golden[f"{tag}/e0"].copy()
    worst = 0.0
    for n in range(1, meta["steps"] + 1):
        e = ora.step(e)
        if n in meta["keep"]:
            ref = golden[f"{tag}/e{n}"]
            err = np.abs(e - ref).max()
            worst = max(worst, err)
            # 1e-12 per step (accumulated linearly) and at most 1e-9 overall
            assert err <= min(1e-9, 1e-12 * n + 1e-13), (tag, n, err)
    obs = ora.observables(e)
    E = golden[f"{tag}/energy"]
    assert abs(obs[0] - E) <= 1e-12 * max(1.0, abs(E))
    assert abs(np.linalg.norm(obs[4:7]) / sc.N - golden[f"{tag}/order"]) <= 1e-13
    assert abs(obs[7] - golden[f"{tag}/torque"]) <= 1e-10 * max(1.0, float(golden[f"{tag}/torque"]))


@pytest.mark.parametrize("tag", ["bcc2_thermal", "sc_open", "sc_tiny_fold", "honeycomb"])
def test_oracle_stencil_csr_equivalent(golden, golden_models, tag):
    """The C neighbour-list builder (used for large supercells) gives the same trajectory."""
    _, meta, a = _oracle(golden_models, tag, "blocks")
    _, _, b = _oracle(golden_models, tag, "stencil")
    ea = golden[f"{tag}/e0"].copy()
    eb = ea.copy()
    for _ in range(meta["steps"]):
        ea, eb = a.step(ea), b.step(eb)
    assert np.abs(ea - eb).max() < 1e-13


@pytest.mark.parametrize("tag", ["sc16", "sc6_thermal", "bcc2_T0", "tri16", "sc_afm"])
def test_oracle_run_table(golden, golden_models, tag):
    """Observable rows of LLGSolver.run (magex/llg.py:254-283) reproduced by stepping the oracle."""
    sc, meta, ora = _oracle(golden_models, tag)
    every = meta["run_every"]
    e = golden[f"{tag}/e0"].copy()
    rows = [ora.row(e)]
    for n in range(1, meta["steps"] + 1):
        e = ora.step(e)
        if n % every == 0 or n == meta["steps"]:
            rows.append(ora.row(e))
    ref = golden[f"{tag}/table"]
    rows = np.array(rows)
    assert rows.shape == ref.shape
    assert np.allclose(rows[:, :6], ref[:, :6], rtol=1e-11, atol=1e-12)
    assert np.allclose(rows[:, 6], ref[:, 6], rtol=1e-9, atol=1e-10)


def test_oracle_larmor(golden, golden_models):
    from magex_gb300.constants import GAMMA
    from magex_gb300.lattice import Supercell
    from magex_gb300.spinmodel import load_results
    sc = Supercell(load_results(golden_models["free"]["model"]), (1, 1, 1), field=(0, 0, 2.0))
    ora = OracleLLG(sc, 0.0, 1e-3)
    e = np.array([[1.0, 0, 0]])
    ph = []
    for _ in range(1000):
        e = ora.step(e)
        ph.append(np.arctan2(e[0, 1], e[0, 0]))
    assert np.abs(e - golden["larmor/e1000"]).max() < 1e-12
    w = np.polyfit(np.arange(1, 1001) * 1e-3, np.unwrap(ph), 1)[0]
    assert abs(abs(w) - GAMMA * 2.0) / (GAMMA * 2.0) < 1e-6


def test_oracle_ziggurat_moments():
    """The port of the reference's parallel normal generator (magex/fast.py:189-200) has the moments
    the reference tests (magex tests/test_fast.py:39-46)."""
    import ctypes as C
    import oracle as O
    lib = O.load()
    n = 300000
    b = np.empty((n, 3))
    st = np.random.SeedSequence(7).generate_state(256, dtype=np.uint64)
    lib.oracle_gauss3(b.ctypes.data_as(C.POINTER(C.c_double)), st.ctypes.data_as(C.POINTER(C.c_uint64)), 256,
                      np.ones(n).ctypes.data_as(C.POINTER(C.c_double)), None, n, 0)
    x = b.ravel()
    assert abs(x.mean()) < 0.006 and abs(x.var() - 1) < 0.006
    assert abs((x ** 4).mean() / x.var() ** 2 - 3) < 0.03
    assert abs((np.abs(x) > 3).mean() / 0.0026998 - 1) < 0.08


def test_oracle_thermal_equilibrium_within_3_sigma_of_reference(golden, golden_models):
    """Equilibrium <E>/N and <|M|> of a Langevin run with the oracle's own (ziggurat) noise stream
    agree with the reference's run (its default_rng stream) within 3 combined standard errors."""
    from helpers import assert_within_3_sigma, block_stats, thermal_system
    sc, th = thermal_system(golden, golden_models)
    ora = OracleLLG(sc, th["alpha"], th["dt"], th["T"], 7, noise="ziggurat", csr="stencil")
    e = sc.init_spins("ferro")
    for _ in range(th["equil"]):
        ora.step_inplace(e)
    E, M = [], []
    for k in range(th["sample"]):
        ora.step_inplace(e)
        if k % th["every"] == th["every"] - 1:
            o = ora.observables(e)
            E.append(o[0] / sc.N)
            M.append(np.linalg.norm(o[1:4]) / sc.N)
    for key, x in (("E", E), ("M", M)):
        assert_within_3_sigma(golden, key, *block_stats(x))


@pytest.mark.parametrize("tag", ["gauss_dmi", "uniform_sc", "heatbath_tri", "hinzke_bcc2", "T0_afm", "open_kagome",
                                 "structure", "bcc2_shell4", "sphere"])
def test_oracle_mc_sweeps_match_reference(golden, golden_models, tag):
    """The oracle's Monte Carlo sweep (same NumPy draws) reproduces magex's MetropolisMC trajectories."""
    from helpers import mc_system
    from oracle import OracleMC
    sc, meta = mc_system(golden, golden_models, tag)
    mc = OracleMC(sc, meta["T"], meta["seed"], meta["sigma"], meta["overrelax"], meta["move"])
    assert np.array_equal(mc.colour, golden[f"mc/{tag}/colour"])
    e = golden[f"mc/{tag}/e0"].copy()
    counts = golden[f"mc/{tag}/accepted_tried"]
    for k in range(1, meta["sweeps"] + 1):
        mc.sweep(e)
        assert np.abs(e - golden[f"mc/{tag}/e{k}"]).max() <= 1e-12, (tag, k)
        assert (mc.accepted, mc.tried) == tuple(int(x) for x in counts[k - 1])


@pytest.mark.parametrize("tag", ["sc_decades", "bcc2_decades"])
def test_oracle_adversarial_trajectory(tag):
    """The adversarial T = 0 fixtures (couplings over eight decades in one stencil, |B| = 100 T, a
    near-zero single-ion term; make_golden.py --adversarial): the oracle follows magex's trajectory
    to 1e-12 per step over 1000 steps, so the fixture is a sound target for the fixed-point sum."""
    import json
    import os
    from magex_gb300.lattice import Supercell
    from magex_gb300.spinmodel import load_results
    adv = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "adversarial.npz"))
    meta = json.loads(str(adv["meta"]))[tag]
    sc = Supercell(load_results(meta["model"], jtol=meta["jtol"]), tuple(meta["L"]), (True, True, True), tuple(meta["B"]))
    ora = OracleLLG(sc, meta["alpha"], meta["dt"], 0.0, 1, csr="stencil", threads=1)
    e = adv[f"{tag}/e0"].copy()
    for n in range(1, meta["keep"][-1] + 1):
        ora.step_inplace(e)
        if n in meta["keep"]:
            err = np.abs(e - adv[f"{tag}/e{n}"]).max()
            assert err <= 1e-12 * n, (tag, n, err)
    E = float(adv[f"{tag}/energy"])
    assert abs(ora.observables(e)[0] - E) <= 1e-12 * abs(E)


def test_config2_thermal_fixture_is_consistent():
    """The reference's config-2 Langevin statistics (make_golden.py --thermal-bcc2): the stored mean
    and errors are those of the stored run means, the first run's stored series gives its run mean,
    and the runs are in the ordered phase they were chosen for (|M| ~ 0.9 at 300 K, below T_c)."""
    import json
    import os
    ref = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "thermal_bcc2.npz"))
    th = json.loads(str(ref["params"]))
    assert len(ref["E_series0"]) == th["sample"] // th["every"]
    for key in ("E", "M"):
        runs = ref[f"{key}_run_means"]
        assert len(runs) == th["nruns"]
        assert abs(runs.mean() - float(ref[f"{key}_mean"])) <= 1e-12 * abs(runs.mean())
        assert abs(runs.std(ddof=1) - float(ref[f"{key}_sd_run"])) <= 1e-9 * runs.std(ddof=1)
        assert abs(ref[f"{key}_series0"].mean() - runs[0]) <= 1e-12 * abs(runs[0])
    assert 0.85 < float(ref["M_mean"]) < 0.97
