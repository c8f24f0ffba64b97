"""Randomised parity: textbook models drawn at random (lattice, shells, DMI, anisotropy, supercell size
down to single cells, open or periodic axes, field, temperature, integrator) stepped by the GB300
kernels and by the oracle with the same host noise.  The oracle is pinned to the reference's own
trajectories (tests/test_oracle_golden.py); here the draws reach shapes the golden cases do not:
tiny periodic supercells where couplings meet their own images, mixed boundaries and several
sublattices with repeated neighbours."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LATTICES = ["chain", "square", "triangular", "honeycomb", "kagome", "sc", "bcc", "fcc"]


def _draw(seed):
    from magex_gb300.lattice import Supercell
    from magex_gb300.spinmodel import load_results, make_model
    rng = np.random.default_rng(seed)
    lat = LATTICES[seed % len(LATTICES)]
    nsh = int(rng.integers(1, 3))
    J = list(np.round(rng.uniform(-1.0, 2.0, nsh), 3))
    D = float(np.round(rng.uniform(0.0, 0.4), 3)) if rng.random() < 0.6 else 0.0
    K = float(np.round(rng.uniform(-0.1, 0.1), 3))
    uc = load_results(make_model(lat, J=J, D=D, K=K, moment=float(rng.choice([1.0, 2.0, 2.5]))))
    dims = {"chain": 1, "square": 2, "triangular": 2, "honeycomb": 2, "kagome": 2}.get(lat, 3)
    L = [int(rng.integers(1, 7)) if a < dims else 1 for a in range(3)]
    pbc = [bool(rng.random() < 0.7) if a < dims else False for a in range(3)]
    B = tuple(np.round(rng.uniform(-1.0, 1.0, 3), 3))
    sc = Supercell(uc, tuple(L), tuple(pbc), B)
    integ = "depondt" if rng.random() < 0.3 else "heun"
    T = float(rng.choice([0.0, 5.0, 50.0]))
    return sc, dict(lattice=lat, J=J, D=D, K=K, L=L, pbc=pbc, B=B, integrator=integ, T=T)


@pytest.mark.parametrize("seed", range(24))
def test_random_model_matches_oracle(cuda, seed):
    from magex_gb300.llg import GB300LLG
    from oracle import OracleLLG
    try:
        sc, meta = _draw(seed)
    except (ValueError, NotImplementedError) as err:       # a draw magex itself refuses
        pytest.skip(f"model not buildable: {err}")
    if sc.N == 0:
        pytest.skip("empty supercell")
    gpu = GB300LLG(sc, 0.1, 1e-3, meta["T"], 7, integrator=meta["integrator"], noise="host")
    ora = OracleLLG(sc, 0.1, 1e-3, meta["T"], 7, integrator=meta["integrator"])
    e0 = sc.init_spins("random", seed=seed)
    a, b = e0.copy(), e0.copy()
    for n in range(1, 6):
        a = gpu.step(a)
        b = ora.step(b)
        assert np.abs(a - b).max() <= 1e-12 * n, (meta, n, np.abs(a - b).max())
    E = ora.observables(b)[0]
    assert abs(gpu.energy(a) - E) <= 1e-12 * max(1.0, abs(E)), meta


def _fixed_eligible(sc):
    return getattr(sc, "A_site", None) is None and getattr(sc, "mu_site", None) is None


@pytest.mark.parametrize("precision", ["fp64_fixed", "int48", "df32"])
@pytest.mark.parametrize("seed", range(24))
def test_random_model_fixed_point_gather_matches_oracle(cuda, seed, precision):
    """The FP64 step with the exact fixed-point exchange sum, and the 48-bit integer and FP32-pair
    forms, on the same random models (the per-sublattice stencil models they accept), at the FP64
    plan's per-step bar."""
    from magex_gb300.llg import GB300LLG
    from oracle import OracleLLG
    try:
        sc, meta = _draw(seed)
    except (ValueError, NotImplementedError) as err:
        pytest.skip(f"model not buildable: {err}")
    if not _fixed_eligible(sc):
        pytest.skip("per-site tensors: the fixed-point form takes per-sublattice models")
    gpu = GB300LLG(sc, 0.1, 1e-3, meta["T"], 7, integrator=meta["integrator"], noise="host", precision=precision)
    ora = OracleLLG(sc, 0.1, 1e-3, meta["T"], 7, integrator=meta["integrator"])
    e0 = sc.init_spins("random", seed=seed)
    a, b = e0.copy(), e0.copy()
    for n in range(1, 6):
        a = gpu.step(a)
        b = ora.step(b)
        assert np.abs(a - b).max() <= 1e-12 * n, (meta, n, np.abs(a - b).max())


@pytest.mark.parametrize("seed", range(24))
def test_random_model_monte_carlo_matches_oracle(cuda, seed):
    """Monte Carlo sweeps with magex's own draws on the random models: the oracle's restatement of
    magex's colour sweep, same colour classes, same accept counts, spins to 1e-11 after 3 sweeps."""
    from magex_gb300.mc import MetropolisMC
    from oracle import OracleMC
    try:
        sc, meta = _draw(seed)
    except (ValueError, NotImplementedError) as err:
        pytest.skip(f"model not buildable: {err}")
    T = max(meta["T"], 5.0)
    move = ("gaussian", "uniform", "heatbath", "hinzke")[seed % 4]
    gpu = MetropolisMC(sc, T, 21, 0.4, seed % 2, move, rng="host")
    ora = OracleMC(sc, T, 21, 0.4, seed % 2, move)
    assert gpu.ncolors == ora.ncolors
    a = sc.init_spins("random", seed=seed)
    b = a.copy()
    for _ in range(3):
        gpu.sweep(a)
        ora.sweep(b)
        assert np.abs(a - b).max() <= 1e-11, (meta, move)
        assert gpu.counts() == (ora.accepted, ora.tried), (meta, move)


def test_random_models_as_one_batch(cuda):
    """The random models that take uniform per-sublattice parameters, stepped together as one batched
    ensemble (mixed lattices, sublattice counts, coupling widths, sizes and boundaries; per-system T
    and seed, Philox and Depondt / Heun as drawn per batch), equal their own plans to 1e-12 per step
    and their energies to 1e-12."""
    from magex_gb300.batched import BatchedLLG
    from magex_gb300.llg import GB300LLG
    systems, Ts, seeds = [], [], []
    for seed in range(24):
        try:
            sc, meta = _draw(seed)
        except (ValueError, NotImplementedError):
            continue
        if sc.alpha_site is None and sc.site_T is None and sc.mu_site is None and len(sc.bond_src):
            systems.append(sc)
            Ts.append(meta["T"])
            seeds.append(100 + seed)
    assert len(systems) >= 12
    for integ in ("heun", "depondt"):
        ens = BatchedLLG(systems, 0.1, 1e-3, Ts, seeds, integrator=integ)
        e0 = [sc.init_spins("random", seed=300 + k) for k, sc in enumerate(systems)]
        ens.set_spins(e0)
        ens.run(8, graph_chunk=0)
        obs = ens.observables()
        for k, sc in enumerate(systems):
            sol = GB300LLG(sc, 0.1, 1e-3, Ts[k], seeds[k], integrator=integ)
            lat = sol.model.to_lattice(e0[k])
            sol.run_lattice(lat, 8)
            err = float((ens.spins(k) - sol.model.from_lattice(lat)).abs().max())
            assert err <= 1e-12 * 8, (k, integ, err)
            E = sol.energy(ens.spins(k).cpu().numpy())
            assert abs(obs[k, 0] - E) <= 1e-12 * max(1.0, abs(E))
