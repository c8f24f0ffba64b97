"""Reduced-FP64 step forms: same parity tolerances as the FP64 kernels.

precision="df32": the exchange sum on FP32 (hi, lo) pairs with error-free TwoProduct / TwoSum steps;
precision="int48": the exchange (and on-site) sum as exact integer arithmetic on 48-bit fixed-point
couplings and spins.  Both keep the spins, the integration and the renormalisation in FP64 and (Heun)
evaluate the rest of the field and the right-hand side on FP32 pairs.  The tests hold them to the FP64
kernels' bars against the reference's trajectories: 1e-12 per step, 1e-9 after 1000 steps.
"""
import numpy as np
import pytest
import torch

from helpers import golden_supercell

pytestmark = pytest.mark.gpu

STENCIL_TRAJ = ["sc16", "sc6_thermal", "bcc2_thermal", "bcc2_T0", "bcc2_shell4", "tri16", "sc_depondt",
                "tri_depondt_thermal", "sc_open", "sc_tiny_fold", "sc_afm", "honeycomb"]


PRECISIONS = ["df32", "int48", "fp64_fixed"]


@pytest.mark.parametrize("precision", PRECISIONS)
@pytest.mark.parametrize("tag", STENCIL_TRAJ)
def test_reduced_trajectory_matches_reference(cuda, golden, golden_models, tag, precision):
    from magex_gb300.llg import GB300LLG
    sc, meta = golden_supercell(golden_models, tag)
    sol = GB300LLG(sc, meta["alpha"], meta["dt"], meta["T"], meta["seed"], integrator=meta["integrator"],
                   noise="host", precision=precision)
    e = golden[f"{tag}/e0"].copy()
    for n in range(1, meta["steps"] + 1):
        e = sol.step(e)
        if n in meta["keep"]:
            err = np.abs(e - golden[f"{tag}/e{n}"]).max()
            assert err <= min(1e-9, 1e-12 * n + 1e-13), (tag, n, err)


@pytest.mark.parametrize("precision", PRECISIONS)
def test_reduced_sc16_1000_steps(cuda, golden, golden_models, precision):
    from magex_gb300.llg import GB300LLG
    sc, meta = golden_supercell(golden_models, "sc16")
    sol = GB300LLG(sc, meta["alpha"], meta["dt"], 0.0, meta["seed"], precision=precision)
    lat = sol.model.to_lattice(golden["sc16/e0"])
    sol.run_lattice(lat, 1000)
    e = sol.model.from_lattice(lat).cpu().numpy()
    assert np.abs(e - golden["sc16/e1000"]).max() <= 1e-9


@pytest.mark.parametrize("precision", PRECISIONS)
def test_reduced_full_size_bcc_against_fp64(cuda, precision):
    """Config-2 lattice (4,194,304 spins, 26 neighbours, full tensors), T = 300 K, same Philox stream:
    20 steps of the reduced plan stay within 1e-12 per step of the FP64 plan."""
    from magex_gb300.llg import GB300LLG
    from magex_gb300.workloads import bcc_two_site
    sc = bcc_two_site(L=128)
    e0 = sc.init_spins("random", seed=5)
    out = []
    for prec in ("fp64", precision):
        sol = GB300LLG(sc, 0.05, 1e-4, 300.0, 77, precision=prec)
        lat = sol.model.to_lattice(e0)
        sol.run_lattice(lat, 20)
        out.append(lat)
    err = float((out[0] - out[1]).abs().max())
    assert err <= 1e-12 * 20, err
    assert float((torch.linalg.vector_norm(out[1], dim=0) - 1).abs().max()) < 1e-14


@pytest.mark.parametrize("integrator", ["heun", "depondt"])
def test_fixed_point_philox_draws_read_back_match_fp64(cuda, integrator):
    """bcc 48^3 (221,184 spins, 26 couplings: the plan runs its stages at five blocks per SM and its
    corrector reads back the predictor's Philox draws), 300 K: 20 steps stay within 1e-12 per step of
    the FP64 plan, which draws the normals in both stages, for both integrators."""
    from magex_gb300.llg import GB300LLG
    from magex_gb300.workloads import bcc_two_site
    sc = bcc_two_site(L=48)
    e0 = sc.init_spins("random", seed=6)
    out = []
    for prec in ("fp64", "fp64_fixed"):
        sol = GB300LLG(sc, 0.05, 1e-4, 300.0, 91, integrator=integrator, precision=prec)
        lat = sol.model.to_lattice(e0)
        sol.run_lattice(lat, 20)
        out.append(lat)
    err = float((out[0] - out[1]).abs().max())
    assert err <= 1e-12 * 20, err


@pytest.mark.parametrize("precision", PRECISIONS)
def test_reduced_refuses_unsupported_layouts(cuda, golden, golden_models, precision):
    from helpers import golden_irregular
    from magex_gb300.llg import GB300LLG
    nl, meta, _ = golden_irregular(golden, golden_models, "sc_sphere")
    with pytest.raises(NotImplementedError):
        GB300LLG(nl, 0.1, 1e-3, precision=precision)


def test_fixed_point_forms_against_fp64_one_step(cuda):
    """bcc 32^3, random spins, one T = 0 step: the 56-bit fixed-point gather with an FP64 tail agrees
    with the FP64 plan at FP64 rounding level, the 48-bit one within its 2^-48 quantisation, the
    compensated-FP32 one within ~2^-44 of the field."""
    from magex_gb300.llg import GB300LLG
    from magex_gb300.workloads import bcc_two_site
    sc = bcc_two_site(L=32)
    e0 = sc.init_spins("random", seed=8)
    out = {}
    for prec in ("fp64", "df32", "int48", "fp64_fixed"):
        sol = GB300LLG(sc, 0.05, 1e-4, 0.0, 1, precision=prec)
        lat = sol.model.to_lattice(e0)
        sol.run_lattice(lat, 1)
        out[prec] = lat
    d_df = float((out["df32"] - out["fp64"]).abs().max())
    d_fx = float((out["int48"] - out["fp64"]).abs().max())
    d_64 = float((out["fp64_fixed"] - out["fp64"]).abs().max())
    assert d_64 <= 1e-15 and d_fx <= 2e-15 and d_df <= 2e-14, (d_64, d_fx, d_df)


@pytest.mark.parametrize("tag", ["sc_cubic", "tri_cubic_thermal"])
def test_fixed_point_sum_with_higher_onsite_terms_matches_reference(cuda, golden, golden_models, tag):
    """The exact fixed-point sum form with cubic (rotated axes) and higher uniaxial anisotropy (its
    HIGHER instantiation: the terms added in FP64 at the site's spin): the reference's trajectories,
    Heun at T = 0 and Depondt at 5 K with the reference's noise stream, at the FP64 bars."""
    from magex_gb300.llg import GB300LLG
    sc, meta = golden_supercell(golden_models, tag)
    sol = GB300LLG(sc, meta["alpha"], meta["dt"], meta["T"], meta["seed"], integrator=meta["integrator"],
                   noise="host", precision="fp64_fixed")
    e = golden[f"{tag}/e0"].copy()
    for n in range(1, meta["steps"] + 1):
        e = sol.step(e)
        if n in meta["keep"]:
            err = np.abs(e - golden[f"{tag}/e{n}"]).max()
            assert err <= min(1e-9, 1e-12 * n + 1e-13), (tag, n, err)
    assert abs(sol.energy(e) - float(golden[f"{tag}/energy"])) <= 1e-12 * abs(float(golden[f"{tag}/energy"]))
