"""Compensated-FP32 exchange gather (precision="df32"): same parity tolerances as the FP64 kernels.

The spins, on-site and Zeeman terms, right-hand side and integration stay FP64; only the exchange sum
is evaluated in FP32 (hi, lo) pairs with error-free TwoProduct / TwoSum steps.  The tests hold it to
the FP64 kernels' bars against the reference's trajectories: 1e-12 per step, 1e-9 after 1000 steps.
"""
import numpy as np
import pytest
import torch

from helpers import golden_supercell

pytestmark = pytest.mark.gpu

STENCIL_TRAJ = ["sc16", "sc6_thermal", "bcc2_thermal", "bcc2_T0", "bcc2_shell4", "tri16", "sc_depondt",
                "tri_depondt_thermal", "sc_open", "sc_tiny_fold", "sc_afm", "honeycomb"]


@pytest.mark.parametrize("tag", STENCIL_TRAJ)
def test_df32_trajectory_matches_reference(cuda, golden, golden_models, tag):
    from magex_gb300.llg import GB300LLG
    sc, meta = golden_supercell(golden_models, tag)
    sol = GB300LLG(sc, meta["alpha"], meta["dt"], meta["T"], meta["seed"], integrator=meta["integrator"],
                   noise="host", precision="df32")
    e = golden[f"{tag}/e0"].copy()
    for n in range(1, meta["steps"] + 1):
        e = sol.step(e)
        if n in meta["keep"]:
            err = np.abs(e - golden[f"{tag}/e{n}"]).max()
            assert err <= min(1e-9, 1e-12 * n + 1e-13), (tag, n, err)


def test_df32_sc16_1000_steps(cuda, golden, golden_models):
    from magex_gb300.llg import GB300LLG
    sc, meta = golden_supercell(golden_models, "sc16")
    sol = GB300LLG(sc, meta["alpha"], meta["dt"], 0.0, meta["seed"], precision="df32")
    lat = sol.model.to_lattice(golden["sc16/e0"])
    sol.run_lattice(lat, 1000)
    e = sol.model.from_lattice(lat).cpu().numpy()
    assert np.abs(e - golden["sc16/e1000"]).max() <= 1e-9


def test_df32_full_size_bcc_against_fp64(cuda):
    """Config-2 lattice (4,194,304 spins, 26 neighbours, full tensors), T = 300 K, same Philox stream:
    20 steps of the df32 plan stay within 1e-12 per step of the FP64 plan."""
    from magex_gb300.llg import GB300LLG
    from magex_gb300.workloads import bcc_two_site
    sc = bcc_two_site(L=128)
    e0 = sc.init_spins("random", seed=5)
    out = []
    for precision in ("fp64", "df32"):
        sol = GB300LLG(sc, 0.05, 1e-4, 300.0, 77, precision=precision)
        lat = sol.model.to_lattice(e0)
        sol.run_lattice(lat, 20)
        out.append(lat)
    err = float((out[0] - out[1]).abs().max())
    assert err <= 1e-12 * 20, err
    assert float((torch.linalg.vector_norm(out[1], dim=0) - 1).abs().max()) < 1e-14


def test_df32_refuses_unsupported_layouts(cuda, golden, golden_models):
    from helpers import golden_irregular
    from magex_gb300.llg import GB300LLG
    nl, meta, _ = golden_irregular(golden, golden_models, "sc_sphere")
    with pytest.raises(NotImplementedError):
        GB300LLG(nl, 0.1, 1e-3, precision="df32")
