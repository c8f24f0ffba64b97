"""GB300 LLG kernels (through the C ABI) against the reference's golden trajectories and the oracle.

Tolerances: spins are unit vectors, so max |e_gpu - e_ref| is a relative error.  Per step the
kernels may differ from the reference by 1e-12 (floating-point summation order and fused
multiply-adds), accumulated linearly; after 1000 T = 0 steps by at most 1e-9.
"""
import numpy as np
import pytest
import torch

from helpers import golden_supercell
from magex_gb300.constants import MU_B

pytestmark = pytest.mark.gpu

TRAJ = ["sc16", "sc6_thermal", "bcc2_thermal", "bcc2_T0", "bcc2_shell4", "tri16", "sc_depondt", "tri_depondt_thermal",
        "sc_open", "sc_tiny_fold", "sc_afm", "honeycomb", "sc_structure", "sc_cubic", "tri_cubic_thermal"]


def _solver(golden_models, tag, noise="host", precision="auto"):
    from magex_gb300.llg import GB300LLG
    sc, meta = golden_supercell(golden_models, tag)
    sol = GB300LLG(sc, meta["alpha"], meta["dt"], meta["T"], meta["seed"], integrator=meta["integrator"], noise=noise,
                   precision=precision)
    return sc, meta, sol


@pytest.mark.parametrize("tag", TRAJ)
def test_trajectory_matches_reference(cuda, golden, golden_models, tag):
    """Every golden trajectory with the default solver (these lattices are small, so precision "auto"
    is the all-FP64 plan; the fixed-point-sum form runs them in tests/test_gpu_df.py)."""
    sc, meta, sol = _solver(golden_models, tag)
    assert sol.precision == "fp64"
    e = golden[f"{tag}/e0"].copy()
    for n in range(1, meta["steps"] + 1):
        e = sol.step(e)
        if n in meta["keep"]:
            err = np.abs(e - golden[f"{tag}/e{n}"]).max()
            assert err <= min(1e-9, 1e-12 * n + 1e-13), (tag, n, err)
    assert abs(sol.energy(e) - float(golden[f"{tag}/energy"])) <= 1e-12 * max(1.0, abs(float(golden[f"{tag}/energy"])))
    assert abs(sol.max_torque(e) - float(golden[f"{tag}/torque"])) <= 1e-10 * max(1.0, float(golden[f"{tag}/torque"]))
    B = sol.effective_field(e)
    ref_B = golden[f"{tag}/field"]
    assert np.abs(B - ref_B).max() <= 1e-12 * max(1.0, np.abs(ref_B).max())
    # the same terms through the system object, as magex's SpinSystem methods
    E = float(golden[f"{tag}/energy"])
    assert abs(sc.energy(e) - E) <= 1e-12 * max(1.0, abs(E))
    assert np.abs(sc.effective_field(e) - ref_B).max() <= 1e-12 * max(1.0, np.abs(ref_B).max())
    ref_g = -MU_B * sc.mu[:, None] * ref_B
    assert np.abs(sc.gradient(e) - ref_g).max() <= 1e-12 * max(1.0, np.abs(ref_g).max())


def test_sc16_1000_steps_device_resident(cuda, golden, golden_models):
    """Config-1 workload: 1000 T = 0 steps kept on the device (one library call), <= 1e-9."""
    from magex_gb300.llg import GB300LLG
    sc, meta = golden_supercell(golden_models, "sc16")
    sol = GB300LLG(sc, meta["alpha"], meta["dt"], 0.0, meta["seed"])
    lat = sol.model.to_lattice(golden["sc16/e0"])
    sol.run_lattice(lat, 1000)
    e = sol.model.from_lattice(lat).cpu().numpy()
    assert np.abs(e - golden["sc16/e1000"]).max() <= 1e-9
    assert abs(sol.time - 0.1) < 1e-12


@pytest.mark.parametrize("tag", ["sc16", "sc6_thermal", "bcc2_T0", "tri16", "sc_afm"])
def test_run_table_matches_reference(cuda, golden, golden_models, tag):
    sc, meta, sol = _solver(golden_models, tag)
    e, tab, snaps = sol.run(golden[f"{tag}/e0"].copy(), meta["steps"], output_every=meta["run_every"], snapshots=2)
    ref = golden[f"{tag}/table"]
    assert tab.shape == ref.shape
    assert np.allclose(tab[:, :6], ref[:, :6], rtol=1e-11, atol=1e-12)
    assert np.allclose(tab[:, 6], ref[:, 6], rtol=1e-9, atol=1e-10)
    assert len(snaps) == 3 and snaps[0][1].shape == (sc.N, 3)


def test_oracle_agrees_on_bcc_32cube_thermal_host_noise(cuda):
    """Config-2 Hamiltonian at 32^3 (65,536 spins), T = 300 K, identical host noise: GPU vs oracle."""
    from magex_gb300.llg import GB300LLG
    from magex_gb300.workloads import bcc_two_site
    from oracle import OracleLLG
    sc = bcc_two_site(L=32)
    e0 = sc.init_spins("random", seed=3)
    gpu = GB300LLG(sc, 0.05, 1e-4, 300.0, 11, noise="host")
    ora = OracleLLG(sc, 0.05, 1e-4, 300.0, 11, csr="stencil")
    a, b = e0.copy(), e0.copy()
    for n in range(1, 6):
        a = gpu.step(a)
        b = ora.step(b)
        assert np.abs(a - b).max() <= 1e-12 * n
    assert abs(gpu.energy(a) - ora.observables(b)[0]) <= 1e-12 * abs(ora.observables(b)[0])


def test_full_size_bcc_128cube_properties(cuda):
    """Config-2 lattice at full size (4,194,304 spins): parity with the oracle for 2 T = 0 steps, unit
    norm after Philox steps, and bit-identical repeat of a seeded Philox run."""
    from magex_gb300.llg import GB300LLG
    from magex_gb300.workloads import bcc_two_site
    from oracle import OracleLLG
    sc = bcc_two_site(L=128)
    e0 = sc.init_spins("random", seed=5)
    gpu = GB300LLG(sc, 0.05, 1e-4, 0.0, 1)
    ora = OracleLLG(sc, 0.05, 1e-4, 0.0, 1, csr="stencil")
    a = gpu.step(gpu.step(e0))
    b = ora.step(ora.step(e0))
    assert np.abs(a - b).max() <= 2e-12
    del ora
    runs = []
    for _ in range(2):
        sol = GB300LLG(sc, 0.05, 1e-4, 300.0, 123)
        lat = sol.model.to_lattice(e0)
        sol.run_lattice(lat, 20)
        runs.append(lat.clone())
    assert torch.equal(runs[0], runs[1])
    norm = torch.linalg.vector_norm(runs[0], dim=0)
    assert float((norm - 1).abs().max()) < 1e-14


def test_topological_charge(cuda, golden):
    from magex_gb300.device import DeviceModel
    from magex_gb300.workloads import triangle_list, triangular_film
    sc = triangular_film(L=30, field=(0, 0, 0))
    dm = DeviceModel(sc)
    dm.set_triangles(*triangle_list(sc))
    for key in ("skyrmion", "random"):
        Q = float(dm.topological_charge(dm.to_lattice(golden[f"topo/{key}_e"])).item())
        assert abs(Q - float(golden[f"topo/{key}_Q"])) < 1e-9, key


def test_larmor_precession(cuda, golden, golden_models):
    from magex_gb300.constants import GAMMA
    from magex_gb300.lattice import Supercell
    from magex_gb300.llg import GB300LLG
    from magex_gb300.spinmodel import load_results
    sc = Supercell(load_results(golden_models["free"]["model"]), (1, 1, 1), field=(0, 0, 2.0))
    sol = GB300LLG(sc, alpha=0.0, dt=1e-3)
    e = np.array([[1.0, 0, 0]])
    ph = []
    for _ in range(1000):
        e = sol.step(e)
        ph.append(np.arctan2(e[0, 1], e[0, 0]))
    assert np.abs(e - golden["larmor/e1000"]).max() < 1e-12
    w = np.polyfit(np.arange(1, 1001) * 1e-3, np.unwrap(ph), 1)[0]
    assert abs(abs(w) - GAMMA * 2.0) / (GAMMA * 2.0) < 1e-6


def test_philox_thermal_equilibrium_langevin(cuda):
    """Free spins in a field at T > 0 with in-kernel Philox noise relax to the classical Langevin
    magnetisation <m_z> = coth(x) - 1/x, x = mu mu_B B / (k_B T) (the reference's test
    tests/test_spindyn.py:77-89 checks the same law with Monte Carlo)."""
    from magex_gb300.constants import K_B, MU_B
    from magex_gb300.lattice import Supercell
    from magex_gb300.llg import GB300LLG
    from magex_gb300.spinmodel import load_results, make_model
    sc = Supercell(load_results(make_model("sc", J=[0.0], moment=2.0)), (16, 16, 16), field=(0, 0, 5.0))
    T = 5.0
    sol = GB300LLG(sc, alpha=0.5, dt=1e-3, temperature=T, seed=9)
    lat = sol.model.to_lattice(sc.init_spins("random", seed=1))
    sol.run_lattice(lat, 8000)
    ms = []
    for _ in range(40):
        sol.run_lattice(lat, 500)
        ms.append(float(lat[2].mean()))
    x = 2.0 * MU_B * 5.0 / (K_B * T)
    assert abs(np.mean(ms) - (1 / np.tanh(x) - 1 / x)) < 0.01


def test_invalid_inputs_raise(cuda, golden_models):
    from magex_gb300.lattice import Supercell
    from magex_gb300.llg import GB300LLG
    from magex_gb300.spinmodel import load_results
    sc = Supercell(load_results(golden_models["sc"]["model"]), (4, 4, 4))
    with pytest.raises(ValueError):
        GB300LLG(sc, dt=-1.0)
    with pytest.raises(ValueError):
        GB300LLG(sc, integrator="leapfrog")
    with pytest.raises(NotImplementedError):
        GB300LLG(sc, integrator="rk4")
    with pytest.raises(NotImplementedError):
        GB300LLG(sc, thermostat="quantum")
    sol = GB300LLG(sc)
    with pytest.raises(ValueError):
        sol.step(np.zeros((3, 3)))


@pytest.mark.parametrize("tag", ["sc_sphere", "sc_interface"])
def test_irregular_lattice_matches_reference(cuda, golden, golden_models, tag):
    """Neighbour-list (CSR) layout: carved sphere with vacancies (thermal, reference noise stream) and
    interface exchange scaling with a pinned layer, against the reference's trajectories."""
    from helpers import golden_irregular
    from magex_gb300.llg import GB300LLG
    nl, meta, _ = golden_irregular(golden, golden_models, tag)
    sol = GB300LLG(nl, meta["alpha"], meta["dt"], meta["T"], meta["seed"], noise="host")
    e = golden[f"{tag}/e0"].copy()
    for _ in range(meta["steps"]):
        e = sol.step(e)
    assert np.abs(e - golden[f"{tag}/e{meta['steps']}"]).max() <= 1e-12 * meta["steps"]
    E = float(golden[f"{tag}/energy"])
    assert abs(sol.energy(e) - E) <= 1e-12 * abs(E)
    assert abs(nl.energy(e) - E) <= 1e-12 * abs(E)
    assert abs(sol.max_torque(e) - float(golden[f"{tag}/torque"])) <= 1e-10 * max(1.0, float(golden[f"{tag}/torque"]))


def test_philox_thermal_equilibrium_within_3_sigma_of_reference(cuda, golden, golden_models):
    """Equilibrium <E>/N and <|M|> with in-kernel Philox noise agree with the reference's own
    Langevin run (default_rng stream, same model, T, alpha, dt and sampling) within 3 combined
    standard errors; two independent Philox seeds are averaged."""
    from helpers import assert_within_3_sigma, block_stats, thermal_system
    from magex_gb300.llg import GB300LLG
    sc, th = thermal_system(golden, golden_models)
    E, M = [], []
    for seed in (5, 6):
        sol = GB300LLG(sc, th["alpha"], th["dt"], th["T"], seed)
        lat = sol.model.to_lattice(sc.init_spins("ferro"))
        sol.run_lattice(lat, th["equil"])
        Es, Ms = [], []
        for _ in range(th["sample"] // th["every"]):
            sol.run_lattice(lat, th["every"])
            o = sol.model.observables(lat).cpu().numpy()
            Es.append(o[0] / sc.N)
            Ms.append(np.linalg.norm(o[1:4]) / sc.N)
        E.append(block_stats(Es))
        M.append(block_stats(Ms))
    for key, st in (("E", E), ("M", M)):
        mean = 0.5 * (st[0][0] + st[1][0])
        sem = 0.5 * np.hypot(st[0][1], st[1][1])
        assert_within_3_sigma(golden, key, mean, sem)


@pytest.mark.parametrize("precision", ["fp64", "fp64_fixed", "df32"])
def test_graph_replayed_run_equals_direct_launches(cuda, precision):
    """run_lattice replays a captured CUDA graph on small lattices (Philox step index read from a
    device counter): bit-identical to launching the steps one by one, also after a field change
    (the graph is re-captured) and across calls that do not start at a chunk boundary."""
    from magex_gb300.llg import GB300LLG
    from magex_gb300.workloads import bcc_two_site
    sc = bcc_two_site(L=6)
    e0 = sc.init_spins("random", seed=9)
    a = GB300LLG(sc, 0.05, 1e-4, 300.0, 4, precision=precision)
    b = GB300LLG(sc, 0.05, 1e-4, 300.0, 4, precision=precision)
    la, lb = a.model.to_lattice(e0), b.model.to_lattice(e0)
    a.run_lattice(la, 70)                          # two 32-step replays + 6 direct steps
    for _ in range(70):
        b.run_lattice(lb, 1)
    assert torch.equal(la, lb)
    for sol in (a, b):
        sol.sc.set_field((0.0, 0.3, 0.2))
    a.run_lattice(la, 64)
    for _ in range(64):
        b.run_lattice(lb, 1)
    assert torch.equal(la, lb)
    for sol in (a, b):                             # new thermal amplitudes: the graph is re-captured
        sol.T = 40.0
    a.run_lattice(la, 64)
    for _ in range(64):
        b.run_lattice(lb, 1)
    assert torch.equal(la, lb)
    # repeated short chunks (tails of 4..63 steps become graphs of their own from the second call on),
    # more step counts than cached graphs, and tails after 32-step replays
    for n in (5, 5, 5, 50, 50, 7, 5, 50, 9, 11, 13, 5, 70, 70, 6, 4, 4, 3, 3):
        a.run_lattice(la, n)
        for _ in range(n):
            b.run_lattice(lb, 1)
        assert torch.equal(la, lb), n


@pytest.mark.parametrize("shells,pbc0,noise,precision,L,extra", [
    ((20.0, 10.0, -1.0), True, "philox", "fp64", (96, 76, 76), None),
    ((20.0, 10.0, -1.0, 1.0), True, "philox", "fp64", (96, 76, 76), None),   # 4th shell: couplings reach 2 layers
    ((20.0, 10.0, -1.0), False, "philox", "fp64", (96, 76, 76), None),        # open along the slab axis
    ((20.0, 10.0, -1.0), True, "host", "fp64", (96, 76, 76), None),
    ((20.0, 10.0, -1.0), True, "philox", "fp64_fixed", (96, 76, 76), None),  # slabs, each split as it lands
    ((20.0, 10.0, -1.0, 1.0), False, "host", "fp64_fixed", (96, 76, 76), None),  # open axis 0, reach 2, host noise
    ((20.0, 10.0, -1.0), True, "philox", "fp64_fixed", (96, 76, 76), "pinned"),   # pinned sites keep their spins
    ((20.0, 10.0, -1.0), True, "philox", "fp64_fixed", (96, 76, 76), "depondt"),
    ((20.0, 10.0, -1.0), True, "philox", "fp64_fixed", (96, 76, 76), "higher"),   # cubic + higher uniaxial
    ((20.0, 10.0, -1.0), True, "philox", "int48", (96, 76, 76), None),
    ((20.0, 10.0, -1.0), True, "philox", "df32", (96, 76, 76), None),        # one piece (reduced split refreshed)
    ((20.0, 10.0, -1.0), True, "philox", "fp64", (4, 512, 256), None),      # four slabs of one layer
    ((20.0, 10.0, -1.0), False, "philox", "fp64", (2, 512, 512), None),     # too thin to split: one piece
])
def test_host_buffer_step_equals_device_step(cuda, shells, pbc0, noise, precision, L, extra):
    """mgx_llg_step_host (pinned host buffers; copies in axis-0 slabs overlapping the stages for FP64
    and fixed-point-gather plans of >= 2^20 sites; the fixed-point slabs packed and split in one pass
    and their correctors writing the (N, 3) rows directly) gives the same bits as the step on device
    spins: also in place, and for pageable numpy input (one piece)."""
    from magex_gb300.lattice import Supercell
    from magex_gb300.llg import GB300LLG
    from magex_gb300.spinmodel import load_results
    from magex_gb300.workloads import bcc_two_site_model
    sc = Supercell(load_results(bcc_two_site_model(J=shells)), L, (pbc0, True, True), (0.0, 0.0, 0.5))
    assert sc.N >= 1 << 20
    rng = np.random.default_rng(9)
    if extra == "pinned":
        sc.pinned = rng.random(sc.N) < 0.05
    if extra == "higher":
        C = np.linalg.qr(rng.normal(size=(3, 3)))[0]
        sc.cubic = (rng.uniform(0.01, 0.05, sc.N), C)
        sc.uniaxial_higher = (rng.uniform(0.0, 0.02, sc.N), rng.uniform(0.0, 0.01, sc.N), np.array([0.0, 0.6, 0.8]))
    integ = "depondt" if extra == "depondt" else "heun"
    a = GB300LLG(sc, 0.05, 1e-4, 300.0, seed=5, noise=noise, precision=precision, integrator=integ)
    b = GB300LLG(sc, 0.05, 1e-4, 300.0, seed=5, noise=noise, precision=precision, integrator=integ)
    e0 = sc.init_spins("random", seed=3)
    h = torch.from_numpy(e0.copy()).pin_memory()
    out = torch.empty_like(h).pin_memory()
    lat = b.model.to_lattice(e0)
    for _ in range(3):
        a.step_host(h, out)
        h, out = out, h
        b.step_lattice(lat)
    assert torch.equal(h, b.model.from_lattice(lat).cpu())
    a.step_host(h, h)
    b.step_lattice(lat)
    assert torch.equal(h, b.model.from_lattice(lat).cpu())
    r = a.step(h.numpy().copy())
    b.step_lattice(lat)
    assert isinstance(r, np.ndarray) and np.array_equal(r, b.model.from_lattice(lat).cpu().numpy())
    assert a.time == pytest.approx(b.time) and a._step_index == b._step_index == 5


@pytest.mark.parametrize("noise", ["philox", "host"])
def test_checkpoint_resume_continues_the_trajectory(cuda, tmp_path, noise):
    """A run stopped after 12 steps, written with checkpoint() and continued by a fresh solver after
    resume() equals 30 uninterrupted steps bit for bit (noise counter, clock and host generator
    restored); a solver with another seed refuses the checkpoint."""
    from magex_gb300.llg import GB300LLG
    from magex_gb300.workloads import bcc_two_site
    sc = bcc_two_site(L=6)
    e0 = sc.init_spins("random", seed=4)
    ref = GB300LLG(sc, 0.05, 1e-4, 300.0, seed=11, noise=noise)
    e = e0
    for _ in range(30):
        e = ref.step(e)
    first = GB300LLG(sc, 0.05, 1e-4, 300.0, seed=11, noise=noise)
    a = e0
    for _ in range(12):
        a = first.step(a)
    path = first.checkpoint(a, str(tmp_path / "ck.npz"))
    second = GB300LLG(sc, 0.05, 1e-4, 0.0, seed=11, noise=noise)     # T comes from the checkpoint
    b = second.resume(path)
    assert second.T == 300.0 and second.time == pytest.approx(12e-4)
    for _ in range(18):
        b = second.step(b)
    assert np.array_equal(b, e)
    assert second.time == pytest.approx(ref.time)
    assert np.abs(sc.init_spins("file", path=path) - a).max() < 1e-15   # also a magex spin file
    with pytest.raises(ValueError):
        GB300LLG(sc, 0.05, 1e-4, 300.0, seed=12, noise=noise).resume(path)


@pytest.mark.parametrize("tag", ["sc_sphere", "sc_interface"])
def test_site_relabelling_gives_the_same_spins(cuda, golden, golden_models, tag):
    """Order / race check: the neighbour-list lattice with its sites relabelled by a random permutation
    (every site keeps its couplings, in the same order, and its per-site data) gives bit-identical
    spins after 20 steps: no kernel result depends on where a site sits in memory or on another
    thread's writes.  The energy, a sum over sites in another order, agrees to rounding."""
    from helpers import golden_irregular
    from magex_gb300.lattice import NeighbourList
    from magex_gb300.llg import GB300LLG
    nl, meta, _ = golden_irregular(golden, golden_models, tag)
    N = nl.N
    perm = np.random.default_rng(5).permutation(N)          # new site k is old site perm[k]
    inv = np.empty(N, np.int64)
    inv[perm] = np.arange(N)
    idx = np.concatenate([np.arange(nl.ptr[i], nl.ptr[i + 1]) for i in perm])
    ptr = np.concatenate([[0], np.cumsum(np.diff(nl.ptr)[perm])])
    pl = NeighbourList(ptr, inv[nl.nbr[idx]], nl.typ[idx], nl.bond_J.reshape(-1, 9), nl.mu[perm], nl.A[perm],
                       nl.signs[perm], nl.B)
    for name in ("pinned", "site_T", "alpha_site"):
        v = getattr(nl, name)
        if v is not None:
            setattr(pl, name, np.asarray(v)[perm])
    a = GB300LLG(nl, meta["alpha"], meta["dt"], 0.0, 1)
    b = GB300LLG(pl, meta["alpha"], meta["dt"], 0.0, 1)
    ea = golden[f"{tag}/e0"].copy()
    eb = ea[perm].copy()
    for _ in range(20):
        ea = a.step(ea)
        eb = b.step(eb)
    assert np.array_equal(eb, ea[perm])
    assert b.energy(eb) == pytest.approx(a.energy(ea), rel=1e-13, abs=1e-12)


@pytest.mark.parametrize("tag", ["pulse", "extra", "both", "sot", "sot_site"])
def test_field_hooks_match_reference(cuda, golden, golden_models, tag):
    """magex's field hooks on the solver (magex/llg.py:124-137), as magex's FMR program and spin-lattice
    coupling use them (magex/programs.py:131, magex/sld.py:171): a uniform field_func(t) whose pulse
    ends between a predictor (t) and its corrector (t + dt), plus a rotating part; an (N, 3)
    field_func(t); a per-site extra_field(e) evaluated at e and at the predicted spins; the spin-orbit
    torque fields (sot=, in-kernel); Heun and Depondt.  Trajectories and the max torque against the
    reference's; run() equals the step loop."""
    from helpers import callable_fields, site_field_func
    from magex_gb300.lattice import Supercell
    from magex_gb300.llg import GB300LLG
    from magex_gb300.spinmodel import load_results
    cal = golden_models["callables"]
    case = cal["cases"][tag]
    ff, xf = callable_fields(cal["params"])
    sc = Supercell(load_results(golden_models[case["model"]]["model"]), case["L"], case["pbc"], case["B"])

    def solver():
        sol = GB300LLG(sc, case["alpha"], case["dt"], 0.0, 3, integrator=case["integrator"],
                       sot=cal["sot"] if case["sot"] else None)
        sol.field_func = {0: None, 1: ff, 2: site_field_func(cal["params"], sc.N)}[int(case["field_func"])]
        sol.extra_field = xf if case["extra_field"] else None
        return sol

    sol = solver()
    e = golden[f"callables/{tag}/e0"].copy()
    for n in range(1, case["steps"] + 1):
        e = sol.step(e)
        if n in case["keep"]:
            err = np.abs(e - golden[f"callables/{tag}/e{n}"]).max()
            assert err <= 1e-12 * n, (tag, n, err)
    tq = float(golden[f"callables/{tag}/torque"])
    assert abs(sol.max_torque(e) - tq) <= 1e-10 * max(1.0, tq)
    e_run, table, _ = solver().run(golden[f"callables/{tag}/e0"].copy(), case["steps"], output_every=case["steps"])
    assert np.array_equal(e_run, e)
    assert table[-1, 6] == pytest.approx(tq, rel=1e-10, abs=1e-10)


@pytest.mark.parametrize("tag", ["pulse", "extra", "both", "sot", "sot_site"])
def test_field_and_rhs_match_reference(cuda, golden, golden_models, tag):
    """LLGSolver.field(e, t) and .rhs(e, b, t) (magex/llg.py:124-151) with every hook, against the
    reference's values at the initial spins."""
    from helpers import callable_fields, site_field_func
    from magex_gb300.lattice import Supercell
    from magex_gb300.llg import GB300LLG
    from magex_gb300.spinmodel import load_results
    cal = golden_models["callables"]
    case = cal["cases"][tag]
    ff, xf = callable_fields(cal["params"])
    sc = Supercell(load_results(golden_models[case["model"]]["model"]), case["L"], case["pbc"], case["B"])
    sol = GB300LLG(sc, case["alpha"], case["dt"], 0.0, 3, integrator=case["integrator"],
                   sot=cal["sot"] if case["sot"] else None)
    sol.field_func = {0: None, 1: ff, 2: site_field_func(cal["params"], sc.N)}[int(case["field_func"])]
    sol.extra_field = xf if case["extra_field"] else None
    e0 = golden[f"callables/{tag}/e0"]
    B, ref_B = sol.field(e0, 0.0), golden[f"callables/{tag}/field0"]
    assert np.abs(B - ref_B).max() <= 1e-12 * max(1.0, np.abs(ref_B).max())
    f, ref_f = sol.rhs(e0, 0.0, 0.0), golden[f"callables/{tag}/rhs0"]
    assert np.abs(f - ref_f).max() <= 1e-12 * max(1.0, np.abs(ref_f).max())


def test_thermal_field_matches_reference(cuda, golden, golden_models):
    """One LLGSolver.thermal_field() draw (magex/llg.py:106-122): same generator, same amplitudes."""
    from magex_gb300.lattice import Supercell
    from magex_gb300.llg import GB300LLG
    from magex_gb300.spinmodel import load_results
    sc = Supercell(load_results(golden_models["sc_dmi"]["model"]), (6, 6, 6), (True, True, True), (0.1, 0, 0.5))
    b = GB300LLG(sc, 0.2, 1e-3, 50.0, 5).thermal_field()
    ref = golden["thermal_field/b"]
    assert np.abs(b - ref).max() <= 1e-14 * np.abs(ref).max()
    assert GB300LLG(sc, 0.2, 1e-3, 0.0, 5).thermal_field() == 0.0


def test_run_stops_on_torque_tol_like_reference(cuda, golden, golden_models):
    """run(torque_tol=...) at T = 0 stops at the first output row whose max torque is below the
    tolerance (magex/llg.py:271-274): same rows, same final spins (AFM relaxation, sc 3^3)."""
    from magex_gb300.lattice import Supercell
    from magex_gb300.llg import GB300LLG
    from magex_gb300.spinmodel import load_results
    sc = Supercell(load_results(golden_models["sc_afm"]["model"]), (3, 3, 3), (True, True, True), (0, 0, 0))
    sol = GB300LLG(sc, 0.5, 2e-3, 0.0, 2)
    e, table, _ = sol.run(golden["run_tol/e0"].copy(), 4000, output_every=100, torque_tol=1e-3)
    ref = golden["run_tol/table"]
    assert table.shape == ref.shape
    assert np.allclose(table[:, :6], ref[:, :6], rtol=1e-9, atol=1e-10)
    assert np.allclose(table[:, 6], ref[:, 6], rtol=1e-6, atol=1e-9)
    assert np.abs(e - golden["run_tol/e"]).max() <= 1e-9


def test_run_callback_and_snapshots_like_reference(cuda, golden, golden_models):
    """A callback sees (n, spins) after every step and may change the temperature for the next one
    (magex's two-temperature hook, magex/llg.py:337-341); snapshots every steps // snapshots.  With
    the reference's noise stream ("host") the table, the callback's view and the final spins equal
    the reference run's."""
    from magex_gb300.lattice import Supercell
    from magex_gb300.llg import GB300LLG
    from magex_gb300.spinmodel import load_results
    sc = Supercell(load_results(golden_models["sc_dmi"]["model"]), (4, 4, 4), (True, True, True), (0.0, 0.0, 0.5))
    sol = GB300LLG(sc, 0.1, 1e-3, 20.0, 8, noise="host")
    seen = []

    def cool(n, e_):
        seen.append([n, float(e_[0, 2])])
        sol.T = 20.0 * np.exp(-0.05 * n)

    e, table, snaps = sol.run(golden["run_cb/e0"].copy(), 40, output_every=10, snapshots=4, callback=cool)
    ref = golden["run_cb/table"]
    assert table.shape == ref.shape
    assert np.allclose(table, ref, rtol=1e-10, atol=1e-11)
    assert np.abs(np.array(seen) - golden["run_cb/seen"]).max() <= 1e-11
    assert np.allclose([t for t, _ in snaps], golden["run_cb/snap_t"], rtol=0, atol=1e-15)
    assert np.abs(snaps[-1][1] - golden["run_cb/snap_last"]).max() <= 1e-11
    assert np.abs(e - golden["run_cb/e"]).max() <= 1e-11


@pytest.mark.parametrize("noise", ["philox", "host"])
def test_every_site_pinned_keeps_the_spins(cuda, golden_models, noise):
    """Edge case: a lattice whose sites are all pinned (magex/structure.py:198-207) keeps its spins bit
    for bit at T > 0, in the step, the graph-replayed run and the host-buffer step; a Monte Carlo plan
    on it has no colour class to update."""
    from magex_gb300.lattice import Supercell
    from magex_gb300.llg import GB300LLG
    from magex_gb300.mc import MetropolisMC
    from magex_gb300.spinmodel import load_results
    sc = Supercell(load_results(golden_models["sc_dmi"]["model"]), (6, 6, 6), (True, True, True), (0.1, 0.0, 0.5))
    sc.pinned = np.ones(sc.N, bool)
    e0 = sc.init_spins("random", seed=2)
    sol = GB300LLG(sc, 0.1, 1e-3, 300.0, 4, noise=noise)
    e = e0.copy()
    for _ in range(3):
        e = sol.step(e)
    assert np.array_equal(e, e0)
    lat = sol.model.to_lattice(e0)
    sol.run_lattice(lat, 70)
    assert np.array_equal(sol.model.from_lattice(lat).cpu().numpy(), e0)
    mc = MetropolisMC(sc, 20.0, seed=1)
    assert mc.ncolors == 0
    f = mc.sweep(e0.copy())
    assert np.array_equal(f, e0) and mc.acceptance() == 0.0


def test_new_entry_points_reject_bad_arguments(cuda, golden_models):
    """Errors of the newer calls surface as the exceptions magex raises (ValueError for bad values,
    NotImplementedError for what the kernels do not offer), with nothing launched."""
    import ctypes as C
    from magex_gb300 import _lib
    from magex_gb300.lattice import Supercell
    from magex_gb300.llg import GB300LLG
    from magex_gb300.mc import MetropolisMC
    from magex_gb300.spinmodel import load_results
    sc = Supercell(load_results(golden_models["sc_dmi"]["model"]), (4, 4, 4), (True, True, True), (0.0, 0.0, 0.5))
    with pytest.raises(NotImplementedError):
        GB300LLG(sc, 0.1, 1e-3, sot=dict(p=[0, 1, 0], B_DL=0.1), precision="fp64_fixed")
    with pytest.raises(NotImplementedError):
        GB300LLG(sc, 0.1, 1e-3, stt=dict(u=[1, 0, 0], beta=0.1))
    sol = GB300LLG(sc, 0.1, 1e-3)
    lib = sol.model.lib
    with pytest.raises(ValueError):                       # p must be a non-zero vector
        _lib.check(lib.mgx_llg_set_sot(sol.handle, _lib.dptr(np.zeros(3)), 0.1, 0.0), "mgx_llg_set_sot")
    fixed = GB300LLG(sc, 0.1, 1e-3, precision="fp64_fixed")
    field = torch.zeros(3 * sc.N, dtype=torch.float64, device="cuda")
    with pytest.raises(NotImplementedError):              # per-site fields: FP64 plans only
        _lib.check(lib.mgx_llg_set_extra_field(fixed.handle, C.c_void_p(field.data_ptr())), "mgx_llg_set_extra_field")
    sol.field_func = lambda t: np.zeros(5)                # neither (3,) nor (N, 3)
    with pytest.raises(ValueError):
        sol.step(sc.init_spins("random", seed=1))
    mc = MetropolisMC(sc, 10.0, seed=1)
    keys = np.array([1, 2], np.uint64)
    with pytest.raises(ValueError):                       # beta must be finite and > 0
        _lib.check(lib.mgx_mc_set_chains(mc.handle, 2, keys.ctypes.data_as(C.c_void_p), _lib.dptr(np.array([1.0, 0.0])),
                                         _lib.dptr(np.array([0.5, 0.5]))), "mgx_mc_set_chains")
    host = MetropolisMC(sc, 10.0, seed=1, rng="host")
    with pytest.raises(NotImplementedError):              # ensembles draw Philox numbers
        _lib.check(lib.mgx_mc_set_chains(host.handle, 2, keys.ctypes.data_as(C.c_void_p), _lib.dptr(np.array([1.0, 1.0])),
                                         _lib.dptr(np.array([0.5, 0.5]))), "mgx_mc_set_chains")
    with pytest.raises(ValueError):
        _lib.check(lib.mgx_mc_chain_counts(mc.handle, C.c_void_p(0), None, None, 0, None), "mgx_mc_chain_counts")


def test_higher_onsite_terms_outside_the_fp64_step_are_refused(cuda, golden_models):
    """Cubic / higher uniaxial anisotropy are in the FP64 step and its fixed-point-sum form (also
    batched), field, observables and Monte Carlo sweep; the reduced forms that do not evaluate them
    refuse such a model instead of dropping the terms."""
    from magex_gb300.llg import GB300LLG
    sc, _ = golden_supercell(golden_models, "sc_cubic")
    assert GB300LLG(sc, 0.1, 1e-3, precision="fp64_fixed").precision == "fp64_fixed"
    GB300LLG(sc, 0.1, 1e-3, precision="fp64")
    for precision in ("df32", "int48"):
        with pytest.raises(NotImplementedError):
            GB300LLG(sc, 0.1, 1e-3, precision=precision)


def test_auto_precision_moves_to_fp64_for_field_hooks(cuda, golden, golden_models):
    """A solver on the default precision ("auto") of an eligible model runs the fixed-point-sum form
    and moves to an FP64 plan, with the same step counter and seed, when a per-site field hook is
    first used; the trajectory then equals an FP64 solver's that used the hook from the start."""
    from magex_gb300.llg import GB300LLG
    from magex_gb300.workloads import bcc_two_site
    sc = bcc_two_site(L=26)                                # 35,152 sites: "auto" picks the fixed-point sum
    e0 = sc.init_spins("random", seed=2)
    a = GB300LLG(sc, 0.05, 1e-4, 300.0, 9)
    b = GB300LLG(sc, 0.05, 1e-4, 300.0, 9, precision="fp64")
    assert a.precision == "fp64_fixed" and b.precision == "fp64"
    ea, eb = a.step(e0), b.step(e0)
    assert np.abs(ea - eb).max() <= 1e-12
    hook = lambda e: 0.3 * np.cross(e, [0.0, 0.0, 1.0])   # noqa: E731  (an extra_field of magex/sld.py:171)
    a.extra_field = hook
    b.extra_field = hook
    for _ in range(3):
        ea, eb = a.step(ea), b.step(eb)
    assert a.precision == "fp64" and a._step_index == b._step_index == 4
    assert np.abs(ea - eb).max() <= 1e-12 * 4
