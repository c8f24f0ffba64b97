"""Slab decomposition on the GB300 (one GPU, slabs exchanging halos through LoopbackTransport): the
split run equals the unsplit GB300LLG run bit for bit (same kernels per site, Philox keyed by the
whole lattice's site index), and the reduced owned-cell observables equal the whole lattice's."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp64", "fp64_fixed", "df32"])
@pytest.mark.parametrize("name,L,pbc,B,world", [
    ("bcc2", (12, 6, 5), (1, 1, 1), (0.0, 0.0, 0.5), 2),
    ("bcc2", (12, 6, 5), (1, 1, 1), (0.0, 0.0, 0.5), 4),
    ("sc_open", (9, 4, 4), (0, 0, 0), (0.2, 0.0, 2.0), 3),
    ("tri_two_shell", (10, 8, 1), (1, 1, 0), (0.0, 0.0, 1.0), 2),
])
def test_slabs_equal_unsplit_run(cuda, golden_models, name, L, pbc, B, world, precision):
    from magex_gb300.lattice import Supercell
    from magex_gb300.llg import GB300LLG
    from magex_gb300.slab import LoopbackTransport, SlabLLG, SlabRun
    from magex_gb300.spinmodel import load_results
    uc = load_results(golden_models[name]["model"])
    alpha, dt, T, seed, steps = 0.1, 1e-4, 150.0, 17, 12
    sc = Supercell(uc, L, pbc, B)
    e0 = sc.init_spins("random", seed=3)
    full = GB300LLG(sc, alpha, dt, T, seed, precision=precision)
    lat = full.model.to_lattice(e0)
    full.run_lattice(lat, steps)
    ref = full.model.from_lattice(lat).cpu().numpy()
    ref_obs = full.model.observables(lat).cpu().numpy()

    slabs = [SlabLLG(uc, L, pbc, B, alpha, dt, T, seed, r, world, precision=precision) for r in range(world)]
    run = SlabRun(slabs, LoopbackTransport())
    lats = [sl.scatter(e0) for sl in slabs]
    run.run(lats, steps)
    split = np.concatenate([sl.owned(x) for sl, x in zip(slabs, lats)])
    assert np.array_equal(split, ref)
    obs = run.observables(lats)
    assert abs(obs[0] - ref_obs[0]) <= 1e-12 * abs(ref_obs[0])
    assert np.abs(obs[1:7] - ref_obs[1:7]).max() <= 1e-12 * sc.N
    assert obs[7] == ref_obs[7]


def test_slab_layer_copy_round_trip(cuda, golden_models):
    """mgx_lattice_layers packs c0 layers of every (component, sublattice) block and writes them back."""
    from magex_gb300.slab import SlabLLG
    from magex_gb300.spinmodel import load_results
    uc = load_results(golden_models["bcc2"]["model"])
    sl = SlabLLG(uc, (8, 3, 2), (1, 1, 1), (0, 0, 0), 0.1, 1e-3, 0.0, 1, 0, 2)
    e0 = np.random.default_rng(1).normal(size=(8 * 3 * 2 * 2, 3))
    lat = sl.scatter(e0)
    L0, L1, L2 = sl.sc.L
    v = lat.view(3, sl.sc.ns, L0, L1 * L2)
    buf = torch.empty(3 * sl.sc.ns * 2 * L1 * L2, dtype=torch.float64, device=lat.device)
    sl._layers("e", lat, 1, 3, buf, True)
    assert torch.equal(buf.view(3, sl.sc.ns, 2, L1 * L2), v[:, :, 1:3])
    lat2 = torch.zeros_like(lat)
    sl._layers("e", lat2, 1, 3, buf, False)
    assert torch.equal(lat2.view(3, sl.sc.ns, L0, L1 * L2)[:, :, 1:3], v[:, :, 1:3])
    assert float(lat2.view(3, sl.sc.ns, L0, L1 * L2)[:, :, 0].abs().max()) == 0.0
