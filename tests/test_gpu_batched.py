"""Batched ensemble (mgx_batch_*) against single-system plans and the oracle."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _ensemble():
    from magex_gb300.lattice import Supercell
    from magex_gb300.spinmodel import load_results, make_model
    from magex_gb300.workloads import bcc_two_site, triangular_film
    systems = [
        triangular_film(L=12, field=(0, 0, 1.0)),
        Supercell(load_results(make_model("triangular", J=[1.0], D=0.3, K=0.05)), (20, 16, 1), (True, True, False),
                  (0.0, 0.0, 2.5)),
        Supercell(load_results(make_model("sc", J=[1.0], D=0.1, K=0.05)), (6, 6, 6), field=(0.1, 0, 0.5)),
        bcc_two_site(L=4),
        Supercell(load_results(make_model("honeycomb", J=[1.0, 0.1], D=0.2, dmi="bulk")), (6, 5, 1),
                  (True, True, False), (0, 0.1, 0.3)),
        Supercell(load_results(make_model("sc", J=[1.0], D=0.2, K=0.1)), (5, 5, 4), (False, False, False),
                  (0.2, 0, 2.0)),
    ]
    T = [5.0, 0.0, 30.0, 300.0, 3.0, 10.0]
    seeds = [11, 12, 13, 14, 15, 16]
    alpha = [0.1, 0.3, 0.2, 0.05, 0.1, 0.15]
    dt = 1e-4
    return systems, T, seeds, alpha, dt


def _singles(systems, T, seeds, alpha, dt, noise="philox"):
    from magex_gb300.llg import GB300LLG
    return [GB300LLG(sc, alpha[k], dt, T[k], seeds[k], noise=noise) for k, sc in enumerate(systems)]


def test_batch_equals_single_system_plans(cuda):
    from magex_gb300.batched import BatchedLLG
    systems, T, seeds, alpha, dt = _ensemble()
    ens = BatchedLLG(systems, alpha, dt, T, seeds)
    e0 = [sc.init_spins("random", seed=100 + k) for k, sc in enumerate(systems)]
    ens.set_spins(e0)
    ens.run(10, graph_chunk=0)
    singles = _singles(systems, T, seeds, alpha, dt)
    for k, sol in enumerate(singles):
        lat = sol.model.to_lattice(e0[k])
        sol.run_lattice(lat, 10)
        ref = sol.model.from_lattice(lat)
        # same per-site code in a different kernel: fused multiply-adds may be contracted differently,
        # so the two agree to round-off (1e-12 per step is the tolerance of every GPU parity test)
        err = float((ens.spins(k) - ref).abs().max())
        assert err <= 1e-12 * 10, (k, err)
    obs = ens.observables()
    for k, sol in enumerate(singles):
        E = sol.energy(ens.spins(k).cpu().numpy())
        assert abs(obs[k, 0] - E) <= 1e-12 * max(1.0, abs(E))


def test_graph_replay_equals_direct_launches(cuda):
    from magex_gb300.batched import BatchedLLG
    systems, T, seeds, alpha, dt = _ensemble()
    e0 = [sc.init_spins("random", seed=200 + k) for k, sc in enumerate(systems)]
    a = BatchedLLG(systems, alpha, dt, T, seeds)
    a.set_spins(e0)
    a.run(23, graph_chunk=0)
    b = BatchedLLG(systems, alpha, dt, T, seeds)
    b.set_spins(e0)
    b.run(10, graph_chunk=5)          # two replays
    b.run(13, graph_chunk=5)          # two replays (same graph) + 3 direct steps
    assert torch.equal(a.e, b.e)


def test_batch_host_noise_matches_oracle(cuda):
    from magex_gb300.batched import BatchedLLG
    from oracle import OracleLLG
    systems, T, seeds, alpha, dt = _ensemble()
    ens = BatchedLLG(systems, alpha, dt, T, seeds, noise="host")
    e0 = [sc.init_spins("random", seed=300 + k) for k, sc in enumerate(systems)]
    ens.set_spins(e0)
    oras = [OracleLLG(sc, alpha[k], dt, T[k], seeds[k]) for k, sc in enumerate(systems)]
    es = [e.copy() for e in e0]
    for n in range(1, 6):
        ens.step()
        for k in range(len(systems)):
            es[k] = oras[k].step(es[k])
            err = np.abs(ens.spins(k).cpu().numpy() - es[k]).max()
            assert err <= 1e-12 * n, (k, n, err)


def test_batch_autotune_keeps_state(cuda):
    from magex_gb300.batched import BatchedLLG
    systems, T, seeds, alpha, dt = _ensemble()
    ens = BatchedLLG(systems, alpha, dt, T, seeds)
    ens.set_spins([sc.init_spins("random", seed=k) for k, sc in enumerate(systems)])
    before = ens.e.clone()
    best, timings = ens.autotune(steps=2)
    assert best in timings and ens.launch == best
    assert torch.equal(ens.e, before)
    ref = BatchedLLG(systems, alpha, dt, T, seeds)
    ref.set_spins([sc.init_spins("random", seed=k) for k, sc in enumerate(systems)])
    ens.run(7, graph_chunk=0)
    ref.run(7, graph_chunk=0)
    assert torch.equal(ens.e, ref.e)           # the launch shape does not change the result


def test_batch_topological_charge(cuda, golden):
    from magex_gb300.batched import BatchedLLG
    from magex_gb300.workloads import triangle_list, triangular_film
    films = [triangular_film(L=30, field=(0, 0, 0)), triangular_film(L=30, field=(0, 0, 1.0))]
    ens = BatchedLLG(films, 0.1, 1e-4, 0.0, [1, 2])
    ens.set_spins([golden["topo/skyrmion_e"], golden["topo/random_e"]])
    ens.set_triangles([triangle_list(sc) for sc in films])
    Q = ens.topological_charge()
    assert abs(Q[0] - float(golden["topo/skyrmion_Q"])) < 1e-9
    assert abs(Q[1] - float(golden["topo/random_Q"])) < 1e-9


def test_film_ensemble_uneven_sizes(cuda):
    """A 24-film slice of the uneven-size ensemble workload: unit norm, finite energies, per-system Q."""
    from magex_gb300.batched import BatchedLLG
    from magex_gb300.workloads import film_ensemble, triangle_list, triangular_film
    spec = film_ensemble(n=24, seed=3)
    films = [triangular_film(L=s["L"], field=s["B"]) for s in spec]
    ens = BatchedLLG(films, 0.1, 1e-4, [s["T"] for s in spec], list(range(24)))
    ens.set_spins([sc.init_spins("random", seed=k) for k, sc in enumerate(films)])
    ens.set_triangles([triangle_list(sc) for sc in films])
    ens.autotune(steps=2)
    ens.run(100)
    norms = torch.linalg.vector_norm(ens.e.view(-1), dim=0)
    assert norms > 0
    for k in range(len(films)):
        blk = ens.block(k)
        assert float((torch.linalg.vector_norm(blk, dim=0) - 1).abs().max()) < 1e-14
    rows = ens.rows()
    assert np.all(np.isfinite(rows)) and rows.shape == (24, 7)
    assert np.all(np.isfinite(ens.topological_charge()))


def test_batch_fp64_fixed_equals_single_system_plans_and_fp64(cuda):
    """The exact fixed-point exchange sum in the batched stages: equal to the single-system plans of the
    same form (same per-site code) and within FP64 rounding of the all-FP64 batch; graph replays are
    bit-identical to direct launches."""
    from magex_gb300.batched import BatchedLLG
    from magex_gb300.llg import GB300LLG
    systems, T, seeds, alpha, dt = _ensemble()
    e0 = [sc.init_spins("random", seed=300 + k) for k, sc in enumerate(systems)]
    fx = BatchedLLG(systems, alpha, dt, T, seeds, precision="fp64_fixed")
    fx.set_spins(e0)
    fx.run(10, graph_chunk=0)
    f64 = BatchedLLG(systems, alpha, dt, T, seeds)
    f64.set_spins(e0)
    f64.run(10, graph_chunk=0)
    for k, sc in enumerate(systems):
        sol = GB300LLG(sc, alpha[k], dt, T[k], seeds[k], precision="fp64_fixed")
        lat = sol.model.to_lattice(e0[k])
        sol.run_lattice(lat, 10)
        ref = sol.model.from_lattice(lat)
        assert float((fx.spins(k) - ref).abs().max()) <= 1e-12 * 10, k
        assert float((fx.spins(k) - f64.spins(k)).abs().max()) <= 1e-12 * 10, k
    g = BatchedLLG(systems, alpha, dt, T, seeds, precision="fp64_fixed")
    g.set_spins(e0)
    g.run(10, graph_chunk=5)
    assert torch.equal(g.e, fx.e)


@pytest.mark.parametrize("precision", ["fp64", "fp64_fixed"])
def test_batch_with_higher_onsite_terms_follows_reference(cuda, golden, golden_models, precision):
    """Cubic (rotated axes) and higher uniaxial anisotropy in batched systems (the HIGHER stage
    instantiation), in both forms: the sc_cubic system (Heun, T = 0) batched with the config-2
    Hamiltonian follows the reference's trajectory and the bcc system its single-system plan; the
    tri_cubic_thermal system (Depondt, 5 K, the reference's noise stream) follows its trajectory."""
    from helpers import golden_supercell
    from magex_gb300.batched import BatchedLLG
    from magex_gb300.llg import GB300LLG
    from magex_gb300.workloads import bcc_two_site
    sc, meta = golden_supercell(golden_models, "sc_cubic")
    bcc = bcc_two_site(L=4)
    ens = BatchedLLG([sc, bcc], [meta["alpha"], 0.05], [meta["dt"], 1e-4], [0.0, 0.0], [meta["seed"], 7],
                     precision=precision)
    e_bcc = bcc.init_spins("random", seed=5)
    ens.set_spins([golden["sc_cubic/e0"], e_bcc])
    ens.run(meta["steps"], graph_chunk=0)
    err = float(np.abs(ens.spins(0).cpu().numpy() - golden[f"sc_cubic/e{meta['steps']}"]).max())
    assert err <= 1e-12 * meta["steps"], err
    single = GB300LLG(bcc, 0.05, 1e-4, 0.0, 7, precision=precision)
    lat = single.model.to_lattice(e_bcc)
    single.run_lattice(lat, meta["steps"])
    assert float((ens.spins(1) - single.model.from_lattice(lat)).abs().max()) <= 1e-12 * meta["steps"]
    sc2, meta2 = golden_supercell(golden_models, "tri_cubic_thermal")
    ens2 = BatchedLLG([sc2], meta2["alpha"], meta2["dt"], meta2["T"], meta2["seed"], integrator="depondt",
                      noise="host", precision=precision)
    ens2.set_spins([golden["tri_cubic_thermal/e0"]])
    ens2.run(meta2["steps"], graph_chunk=0)
    err2 = float(np.abs(ens2.spins(0).cpu().numpy() - golden[f"tri_cubic_thermal/e{meta2['steps']}"]).max())
    assert err2 <= 1e-12 * meta2["steps"], err2
