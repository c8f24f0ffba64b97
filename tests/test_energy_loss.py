"""The differentiable energy loss of the adjoint module (CPU): equal to the oracle's energy and to
central differences in the shell tensors."""
import numpy as np
import torch

from oracle import OracleLLG


def _setup():
    from magex_gb300.adjoint import CouplingGroups
    from magex_gb300.workloads import bcc_two_site, uniaxial_sia
    sc = bcc_two_site(L=3, J=(20.0, 10.0, -1.0, 1.0), dmi_frac=0.05, per="shell", seed=1, field=(0, 0, 0.3))
    groups = CouplingGroups.per_shell(sc)
    T = torch.as_tensor(groups.tensors_from(sc))
    A = torch.as_tensor(np.stack([uniaxial_sia(0.01)] * sc.ns))
    B = torch.tensor([0.0, 0.0, 0.3], dtype=torch.float64)
    return sc, groups, T, A, B


def test_energy_per_site_sums_to_the_oracle_energy():
    from magex_gb300.adjoint import energy_per_site
    sc, groups, T, A, B = _setup()
    e = sc.init_spins("random", seed=3)
    E = float(energy_per_site(sc, groups, torch.as_tensor(e), T, A, B).sum())
    ref = OracleLLG(sc, csr="stencil").observables(e)[0]
    assert abs(E - ref) <= 1e-12 * abs(ref)


def test_energy_gradient_in_shell_tensors_matches_central_differences():
    from magex_gb300.adjoint import energy_per_site
    sc, groups, T, A, B = _setup()
    e = torch.as_tensor(sc.init_spins("random", seed=4))
    Tg = T.clone().requires_grad_(True)
    energy_per_site(sc, groups, e, Tg, A, B).mean().backward()
    h = 1e-5
    for s, a, b in [(0, 0, 0), (1, 0, 2), (2, 2, 1), (3, 1, 1)]:
        Tp, Tm = T.clone(), T.clone()
        Tp[s, a, b] += h
        Tm[s, a, b] -= h
        fd = (energy_per_site(sc, groups, e, Tp, A, B).sum() - energy_per_site(sc, groups, e, Tm, A, B).sum())
        fd = float(fd) / sc.N / (2 * h)
        assert abs(fd - float(Tg.grad[s, a, b])) <= 1e-8 * max(1.0, abs(fd)), (s, a, b)
