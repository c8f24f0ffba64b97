"""S(q, w) sampling on the GB300 against the reference (magex/spectra.py:49-84).

* the device Fourier projection equals magex's dense phase-matrix product ph^T e (to 1e-12 of |m_q|)
  for commensurate and incommensurate q on 1-, 2- and 3-dimensional supercells;
* structure_factor with the reference's own noise stream reproduces magex's S_perp, S_par, energy
  grid and final spins.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _dense_mq(sc, e, qfrac):
    B = 2 * np.pi * np.linalg.inv(np.asarray(sc.uc.cell, float)).T
    qc = np.asarray(qfrac, float) @ B
    ph = np.exp(-1j * sc.positions @ qc.T) / np.sqrt(sc.N)
    return ph.T @ e


@pytest.mark.parametrize("name,L,pbc", [("tri", (8, 8, 1), (1, 1, 0)), ("bcc2", (5, 4, 3), (1, 1, 1)),
                                        ("honeycomb_bulk", (6, 5, 1), (1, 1, 0)), ("sc_open", (7, 3, 5), (0, 0, 0))])
def test_projection_matches_dense_phase_product(cuda, golden_models, name, L, pbc):
    from magex_gb300.device import DeviceModel
    from magex_gb300.lattice import Supercell
    from magex_gb300.spectra import FourierProjector
    from magex_gb300.spinmodel import load_results
    sc = Supercell(load_results(golden_models[name]["model"]), L, tuple(bool(p) for p in pbc))
    rng = np.random.default_rng(3)
    qfrac = np.concatenate([rng.integers(-4, 5, size=(6, 3)) / np.array(L), rng.uniform(-1, 1, size=(5, 3))])
    e = sc.init_spins("random", seed=5)
    dm = DeviceModel(sc)
    proj = FourierProjector(dm, qfrac)
    got = proj.project(dm.to_lattice(e)).cpu().numpy()
    ref = _dense_mq(sc, e, qfrac)
    assert np.abs(got - ref).max() <= 1e-12 * max(1.0, np.abs(ref).max())


@pytest.mark.parametrize("tag,uc", [("tri", "tri"), ("bcc2", "bcc2")])
def test_structure_factor_matches_reference(cuda, golden, golden_models, tag, uc):
    from magex_gb300.lattice import Supercell
    from magex_gb300.llg import GB300LLG
    from magex_gb300.spectra import structure_factor
    from magex_gb300.spinmodel import load_results
    m = golden_models["sqw__" + tag]
    sc = Supercell(load_results(golden_models[uc]["model"]), tuple(m["L"]), tuple(m["pbc"]), tuple(m["B"]))
    sol = GB300LLG(sc, m["alpha"], m["dt"], m["T"], m["seed"], noise="host")
    E, Sp, Sl, e = structure_factor(sc, sol, golden[f"sqw/{tag}/e0"].copy(), np.array(m["qfrac"]), m["nsteps"],
                                    m["sample_every"], m["nseg"])
    assert np.allclose(E, golden[f"sqw/{tag}/E"], rtol=1e-13, atol=0)
    for got, key in ((Sp, "S_perp"), (Sl, "S_par")):
        ref = golden[f"sqw/{tag}/{key}"]
        assert got.shape == ref.shape
        assert np.abs(got - ref).max() <= 1e-8 * np.abs(ref).max(), key
    assert np.abs(e - golden[f"sqw/{tag}/e_end"]).max() <= 1e-10


def test_projection_large_lattice_properties(cuda):
    """bcc 64^3 (524,288 spins): a uniform state projects onto q = 0 only (|m_0| = sqrt(N) |e|), and
    a single reciprocal-lattice shift of q leaves m_q unchanged up to the sublattice phase."""
    from magex_gb300.device import DeviceModel
    from magex_gb300.spectra import FourierProjector
    from magex_gb300.workloads import bcc_two_site
    sc = bcc_two_site(L=64)
    dm = DeviceModel(sc)
    q = np.array([[0, 0, 0], [1 / 64, 0, 0], [0.25, 0.5, 0.125], [1.25, 0.5, 0.125]])
    proj = FourierProjector(dm, q)
    lat = dm.to_lattice(np.tile([0.6, 0.0, 0.8], (sc.N, 1)))
    m = proj.project(lat).cpu().numpy()
    assert abs(m[0, 2] - 0.8 * np.sqrt(sc.N)) < 1e-9
    assert np.abs(m[1:3]).max() < 1e-9
    lat = dm.to_lattice(sc.init_spins("random", seed=2))
    m = proj.project(lat).cpu().numpy()
    pos = np.asarray(sc.uc.positions).reshape(sc.ns, 3)
    assert np.abs(m[2]).max() > 1e-3                           # a generic state has weight at q
    ref = _dense_mq_sub(sc, lat, q[2:], pos)
    assert np.abs(m[2:] - ref).max() <= 1e-10 * np.abs(ref).max()


def _dense_mq_sub(sc, lat, q, pos):
    """m_q from per-sublattice 3D FFTs (torch) as an independent check at large N."""
    B = 2 * np.pi * np.linalg.inv(np.asarray(sc.uc.cell, float)).T
    e = lat.reshape(3, sc.ns, *sc.L)
    F = torch.fft.fftn(e.to(torch.complex128), dim=(2, 3, 4)).cpu().numpy()
    out = []
    for qf in q:
        k = np.mod(np.round(qf * np.array(sc.L)).astype(int), sc.L)
        ph = np.exp(-1j * pos @ (qf @ B))
        out.append(sum(ph[s] * F[:, s, k[0], k[1], k[2]] for s in range(sc.ns)) / np.sqrt(sc.N))
    return np.array(out)
