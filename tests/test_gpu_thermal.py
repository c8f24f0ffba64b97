"""Thermal equilibrium of the benchmark Hamiltonian against the reference's own Langevin run.

The fixture (tests/golden/thermal_bcc2.npz, written by make_golden.py --thermal-bcc2) holds the
equilibrium <E>/N and <|M|> of magex's LLGSolver (NumPy Heun, its default_rng noise stream,
magex/llg.py:106-122,216-227) on the two-site bcc model with full 3x3 tensors, DMI, SIA and
B_z = 0.5 T at 300 K (8^3 cells), from 20 block means.  The GPU runs the same model, parameters and
sampling with in-kernel Philox noise (FP32 Box-Muller of Philox4x32-10 draws), in every step form,
and must land within 3 combined standard errors; magex checks its own thermostat the same way against
a known law (tests/test_spindyn.py:79-89).  A run at a temperature 10 % off must fail the same bound,
so the check can tell a wrong noise amplitude from a right one.
"""
import json
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def ref():
    return np.load(os.path.join(HERE, "golden", "thermal_bcc2.npz"))


def _system(th):
    from magex_gb300.workloads import bcc_two_site
    return bcc_two_site(L=th["L"], field=(0.0, 0.0, th["Bz"]))


def _stats(sc, th, precision, seeds, T=None):
    """Means and standard errors of E/N and |M| over `seeds` independent Philox runs, each sampled
    as the reference run was (ferromagnetic start, equil steps, then every `every` steps)."""
    from helpers import block_stats
    from magex_gb300.llg import GB300LLG
    out = {"E": [], "M": []}
    for seed in seeds:
        sol = GB300LLG(sc, th["alpha"], th["dt"], th["T"] if T is None else T, seed, precision=precision)
        lat = sol.model.to_lattice(sc.init_spins("ferro"))
        sol.run_lattice(lat, th["equil"])
        obs = []
        for _ in range(th["sample"] // th["every"]):
            sol.run_lattice(lat, th["every"])
            obs.append(sol.model.observables(lat).clone())
        o = torch.stack(obs).cpu().numpy()
        out["E"].append(block_stats(o[:, 0] / sc.N))
        out["M"].append(block_stats(np.linalg.norm(o[:, 1:4], axis=1) / sc.N))
    res = {}
    for key, st in out.items():
        mean = float(np.mean([m for m, _ in st]))
        sem = float(np.sqrt(np.sum([s ** 2 for _, s in st]))) / len(st)
        res[key] = (mean, sem)
    return res


def _sigmas(ref, key, mean, sem):
    return abs(mean - float(ref[f"{key}_mean"])) / np.hypot(float(ref[f"{key}_sem"]), sem)


@pytest.mark.parametrize("precision", ["fp64", "fp64_fixed", "int48", "df32"])
def test_config2_thermal_equilibrium_within_3_sigma_of_reference(cuda, ref, precision):
    th = json.loads(str(ref["params"]))
    sc = _system(th)
    res = _stats(sc, th, precision, seeds=(101, 202))
    for key in ("E", "M"):
        z = _sigmas(ref, key, *res[key])
        assert z <= 3.0, (precision, key, res[key], float(ref[f"{key}_mean"]), float(ref[f"{key}_sem"]), z)


def test_config2_thermal_check_fails_at_10_percent_wrong_temperature(cuda, ref):
    """The same comparison at 0.9 T and 1.1 T: <E>/N moves by tens of standard errors, far outside
    the 3-sigma bound, so a noise amplitude off by 5 % (T off by 10 %) cannot pass."""
    th = json.loads(str(ref["params"]))
    sc = _system(th)
    for factor in (0.9, 1.1):
        res = _stats(sc, th, "fp64", seeds=(101, 202), T=factor * th["T"])
        z = _sigmas(ref, "E", *res["E"])
        assert z > 10.0, (factor, res["E"], z)
