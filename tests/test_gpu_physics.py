"""Physics pins of the reference's LLG tests, run through the GB300 kernels.

Each test states the same law on the same kind of system as the reference's unit test named in its
docstring: the field is minus the energy gradient (finite differences), energy conservation without
damping, relaxation to the antiferromagnetic ground state with damping, Larmor precession of both
integrators, and the integrators the kernels do not implement being refused."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _supercell(lattice, L, field=(0.0, 0.0, 0.0), pbc=(True, True, True), **kw):
    from magex_gb300.lattice import Supercell
    from magex_gb300.spinmodel import load_results, make_model
    return Supercell(load_results(make_model(lattice, **kw)), L, pbc, field)


@pytest.mark.parametrize("precision", ["fp64", "fp64_fixed"])
def test_field_is_minus_energy_gradient(cuda, precision):
    """B_eff = -(dE/de) / (mu mu_B) against central differences of the device energy, h = 1e-6
    (tests/test_spindyn.py:23-33: two shells, interfacial DMI, single-ion anisotropy, oblique field)."""
    from magex_gb300.constants import MU_B
    from magex_gb300.llg import GB300LLG
    sc = _supercell("triangular", (5, 5, 1), field=(0.1, 0.2, 0.5), J=[1.0, 0.2], D=0.3, K=0.1)
    sol = GB300LLG(sc, alpha=0.1, dt=1e-4, precision=precision)
    e = sc.init_spins("random", seed=1)
    g = -sol.effective_field(e) * (sc.mu[:, None] * MU_B)
    h = 1e-6
    for i, a in [(0, 0), (3, 2), (7, 1), (24, 0)]:
        ep, em = e.copy(), e.copy()
        ep[i, a] += h
        em[i, a] -= h
        fd = (sol.energy(ep) - sol.energy(em)) / (2 * h)
        assert abs(fd - g[i, a]) < 1e-6 * max(1.0, abs(fd)), (i, a, fd, g[i, a])


@pytest.mark.parametrize("integrator", ["heun", "depondt"])
def test_energy_conserved_without_damping(cuda, integrator):
    """alpha = 0: the energy drifts by less than 1e-4 (relative) over 500 steps
    (tests/test_spindyn.py:48-55: sc 4^3, J = 1 meV, K = 0.05 meV, dt = 0.2 fs)."""
    from magex_gb300.llg import GB300LLG
    sc = _supercell("sc", (4, 4, 4), J=[1.0], K=0.05)
    e = sc.init_spins("random", seed=3)
    sol = GB300LLG(sc, alpha=0.0, dt=2e-4, integrator=integrator)
    E0 = sol.energy(e)
    for _ in range(500):
        e = sol.step(e)
    assert abs(sol.energy(e) - E0) / abs(E0) < 1e-4
    assert np.abs(np.linalg.norm(e, axis=1) - 1.0).max() < 1e-12


def test_damping_reaches_antiferromagnetic_ground_state(cuda):
    """alpha = 0.5 relaxes a perturbed Neel state to order parameter > 0.999 within 4000 steps
    (tests/test_spindyn.py:58-63: sc 3^3 of the two-site AFM cell, J = -1 meV, cone 0.3)."""
    from magex_gb300.llg import GB300LLG
    sc = _supercell("sc", (3, 3, 3), J=[-1.0], order="afm")
    e = sc.init_spins("reference", cone=0.3, seed=2)
    sol = GB300LLG(sc, alpha=0.5, dt=2e-3)
    e, table, _ = sol.run(e, 4000, output_every=500)
    assert sc.order_parameter(e) > 0.999
    assert table[-1, 5] == pytest.approx(sc.order_parameter(e), abs=1e-12)
    assert np.all(np.diff(table[:, 1]) <= 1e-12)        # damping never raises the energy


@pytest.mark.parametrize("integrator", ["heun", "depondt"])
def test_integrators_larmor(cuda, integrator):
    """A free spin precesses at gamma B with its z component fixed (tests/test_universal.py:109-118:
    B = 1 T, alpha = 0, 1000 steps of 1 fs, e0 = (1, 0, 0.3) / |.|)."""
    from magex_gb300.constants import GAMMA
    from magex_gb300.llg import GB300LLG
    sc = _supercell("sc", (1, 1, 1), field=(0.0, 0.0, 1.0), pbc=(False, False, False), J=[0.0])
    e = np.array([[1.0, 0.0, 0.3]]) / np.sqrt(1.09)
    sol = GB300LLG(sc, alpha=0.0, dt=1e-3, integrator=integrator)
    for _ in range(1000):
        e = sol.step(e)
    assert abs(np.arctan2(e[0, 1], e[0, 0]) - GAMMA * 1.0) < 1e-4
    assert abs(e[0, 2] - 0.3 / np.sqrt(1.09)) < 1e-4


@pytest.mark.parametrize("integrator", ["rk4", "sib", "euler"])
def test_other_integrators_are_refused(cuda, integrator):
    """magex's NumPy path also offers rk4 / sib / euler (magex/llg.py:45); like its CUDA backend
    (magex/cuda_backend.py:315-316) the GB300 solver refuses what its kernels do not implement."""
    from magex_gb300.llg import GB300LLG
    sc = _supercell("sc", (2, 2, 2), J=[1.0])
    with pytest.raises(NotImplementedError):
        GB300LLG(sc, alpha=0.1, dt=1e-3, integrator=integrator)
