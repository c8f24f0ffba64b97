"""Thermal equilibrium of the benchmark Hamiltonian against the reference's own Langevin runs.

The fixture (tests/golden/thermal_bcc2.npz, written by make_golden.py --thermal-bcc2) holds the
equilibrium <E>/N and <|M|> of eight independent runs of magex's LLGSolver (NumPy Heun, its
default_rng noise stream, magex/llg.py:106-122,216-227) on the two-site bcc model with full 3x3
tensors, DMI, SIA and B_z = 0.5 T at 300 K (8^3 cells): per run the mean over 10,000 samples, and
the scatter of those run means (sd_run).  The GPU runs the same model, parameters, run length and
sampling with in-kernel Philox noise (FP32 Box-Muller of Philox4x32-10 draws), in every step form,
with four seeds (two for the reduced forms); under the hypothesis that it samples the same
distribution its run means scatter like the reference's, so the difference of the two averages is
compared with 3 sd_run sqrt(1/8 + 1/n).  magex checks its own thermostat the same way against a known law
(tests/test_spindyn.py:79-89).  Runs at a temperature 10 % off must fail the same bound, so the
check tells a wrong noise amplitude from a right one.
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


def _run_means(sc, th, precision, seeds, temps=None):
    """Per-run means of E/N and |M| of Philox runs sampled as the reference runs were (ferromagnetic
    start, `equil` steps, then a sample every `every` steps over `sample` steps).  Runs k = (seed,
    temperature) pairs; the FP64 forms advance all of them as one batched ensemble (each system
    evolves as a single-system plan with its seed would), the reduced forms one by one."""
    from magex_gb300.batched import BatchedLLG
    from magex_gb300.llg import GB300LLG
    temps = [th["T"]] * len(seeds) if temps is None else list(temps)
    nrun = len(seeds)
    nsamp = th["sample"] // th["every"]
    if precision in ("fp64", "fp64_fixed"):
        ens = BatchedLLG([sc] * nrun, th["alpha"], th["dt"], temps, list(seeds), precision=precision)
        ens.set_spins([sc.init_spins("ferro")] * nrun)
        ens.run(th["equil"], graph_chunk=100)
        obs = np.empty((nsamp, nrun, 8))
        for k in range(nsamp):
            ens.run(th["every"], graph_chunk=th["every"])
            obs[k] = ens.observables()
    else:
        obs = np.empty((nsamp, nrun, 8))
        for r, (seed, T) in enumerate(zip(seeds, temps)):
            sol = GB300LLG(sc, th["alpha"], th["dt"], T, seed, precision=precision)
            lat = sol.model.to_lattice(sc.init_spins("ferro"))
            sol.run_lattice(lat, th["equil"])
            rows = []
            for _ in range(nsamp):
                sol.run_lattice(lat, th["every"])
                rows.append(sol.model.observables(lat).clone())
            obs[:, r] = torch.stack(rows).cpu().numpy()
    E = obs[:, :, 0].mean(0) / sc.N
    M = (np.linalg.norm(obs[:, :, 1:4], axis=2) / sc.N).mean(0)
    return {"E": E, "M": M}


SEEDS = (101, 202, 303, 404)


def _z(ref, key, means):
    """Difference of the GPU and reference averages in units of its standard error (the run-mean
    scatter sd_run of the reference runs, shared by runs of the same length)."""
    n_ref = len(ref[f"{key}_run_means"])
    se = float(ref[f"{key}_sd_run"]) * np.sqrt(1.0 / n_ref + 1.0 / len(means))
    return abs(float(np.mean(means)) - float(ref[f"{key}_mean"])) / se


@pytest.mark.parametrize("precision", ["fp64", "fp64_fixed", "int48", "df32"])
def test_config2_thermal_equilibrium_within_3_sigma_of_reference(cuda, ref, precision):
    th = json.loads(str(ref["params"]))
    sc = _system(th)
    means = _run_means(sc, th, precision, SEEDS if precision in ("fp64", "fp64_fixed") else SEEDS[:2])
    for key in ("E", "M"):
        z = _z(ref, key, means[key])
        assert z <= 3.0, (precision, key, means[key].tolist(), float(ref[f"{key}_mean"]), z)


def test_config2_thermal_check_fails_at_10_percent_wrong_temperature(cuda, ref):
    """The same comparison at 0.9 T and 1.1 T: <E>/N moves by about 2.8 meV, tens of standard errors,
    far outside the 3-sigma bound, so a noise amplitude off by 5 % (T off by 10 %) cannot pass."""
    th = json.loads(str(ref["params"]))
    sc = _system(th)
    means = _run_means(sc, th, "fp64_fixed", SEEDS[:2] * 2, temps=[0.9 * th["T"]] * 2 + [1.1 * th["T"]] * 2)
    for k, factor in enumerate((0.9, 1.1)):
        z = _z(ref, "E", means["E"][2 * k:2 * k + 2])
        assert z > 10.0, (factor, means["E"].tolist(), z)
