"""Adjoint of the Heun step (mgx_adjoint_*, magex_gb300.adjoint) against torch autograd of a dense
FP64 restatement and against central finite differences.

The reference has no gradients, so parity is pinned by these two independent derivatives of the
same forward trajectory.  Parameterisation of the differentiable-LLG workload: J_b = J1 I + D S_b
(S_b = skew(n x r_b)), A = -K (z z^T - I/3), B = (0, 0, B_z); loss = sum_i |e_i(T) - e_target_i|^2
with the target from a second seeded run at perturbed (J1, D, K, B_z).
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

J1, D, K, BZ, ALPHA, DT = 1.0, 0.3, 0.05, 2.0, 0.3, 1e-4


def _params(theta, S):
    """(T (ngroups,3,3), A (1,3,3), B (3)) torch tensors from theta = (J1, D, K, Bz); S holds the DMI basis
    matrix of each coupling group (its canonical coupling)."""
    j1, d, k, bz = theta[0], theta[1], theta[2], theta[3]
    eye = torch.eye(3, dtype=torch.float64, device=theta.device)
    T = j1 * eye[None] + d * S
    zz = torch.zeros((3, 3), dtype=torch.float64, device=theta.device)
    zz[2, 2] = 1.0
    A = (-k * (zz - eye / 3.0))[None]
    B = torch.stack([torch.zeros_like(bz), torch.zeros_like(bz), bz])
    return T, A, B


def _setup(L, nsteps, seg, precision="auto"):
    from magex_gb300.adjoint import AdjointLLG
    from magex_gb300.workloads import film_parameter_basis, triangular_film
    sc = triangular_film(L=L, field=(0, 0, BZ))
    adj = AdjointLLG(sc, alpha=ALPHA, dt=DT, seg_steps=seg, precision=precision)
    S = torch.as_tensor(group_basis(adj, film_parameter_basis(sc)), dtype=torch.float64)
    assert adj.groups.ngroups == 3                      # 6 nearest neighbours = 3 reverse pairs
    assert np.allclose(adj.T0, (J1 * np.eye(3)[None] + D * S.numpy()), atol=1e-15)
    return sc, adj, S


def group_basis(adj, S_bond):
    """Per-group DMI basis from the per-coupling one (the group tensor is its canonical coupling's)."""
    G = adj.groups
    out = np.zeros((G.ngroups, 3, 3))
    for b in range(len(G.group)):
        if not G.transposed[b]:
            out[G.group[b]] = S_bond[b]
    return out


def _loss_and_grads(adj, S, e0, target, theta0, nsteps):
    from magex_gb300.adjoint import llg_trajectory
    theta = torch.tensor(theta0, dtype=torch.float64, requires_grad=True)
    e = torch.as_tensor(e0, dtype=torch.float64, device=adj.device).clone().requires_grad_(True)
    T, A, B = _params(theta, S)
    eT = llg_trajectory(adj, e, T, A, B, nsteps)
    loss = ((eT - target) ** 2).sum()
    loss.backward()
    return float(loss.detach()), theta.grad.numpy().copy(), e.grad.detach().cpu().numpy()


def _central_difference(e_plus, e_minus, target, h):
    """(L(+h) - L(-h)) / 2h for L = sum |e - t|^2, evaluated as sum (e+ - e-).(e+ + e- - 2t) / 2h: the
    same central difference without subtracting two large sums (which would cost ~1e-5 relative)."""
    d = (e_plus - e_minus) * (e_plus + e_minus - 2.0 * target)
    return float(np.sum(d.double().cpu().numpy(), dtype=np.float64)) / (2.0 * h)


def _target(adj, S, sc, nsteps):
    from magex_gb300.adjoint import llg_trajectory
    tt = torch.tensor([1.1 * J1, 0.8 * D, 1.5 * K, 0.7 * BZ], dtype=torch.float64)
    T, A, B = _params(tt, S)
    e1 = torch.as_tensor(sc.init_spins("random", seed=2), device=adj.device)
    with torch.no_grad():
        return llg_trajectory(adj, e1, T, A, B, nsteps).detach()


@pytest.mark.parametrize("precision", ["fp64", "fp64_fixed"])
def test_adjoint_matches_torch_autograd_16x16(cuda, precision):
    """Gradient w.r.t. e(0), J1, D, K, B_z of a 300-step trajectory (checkpoints every 40 steps)
    equals torch autograd through the dense FP64 restatement on a 16 x 16 film, with the forward and
    its recomputation in the FP64 form and in the form with the exact fixed-point exchange sum."""
    from torch_reference import coupling_index, heun_trajectory
    nsteps = 300
    sc, adj, S = _setup(16, nsteps, 40, precision)
    assert adj.precision == precision
    target = _target(adj, S, sc, nsteps)
    e0 = sc.init_spins("random", seed=1)
    theta0 = [J1, D, K, BZ]
    L_gpu, g_gpu, ge_gpu = _loss_and_grads(adj, S, e0, target, theta0, nsteps)

    idx = coupling_index(sc)
    theta = torch.tensor(theta0, dtype=torch.float64, requires_grad=True)
    e = torch.as_tensor(e0).clone().requires_grad_(True)
    T, A, B = _params(theta, S)
    eT = heun_trajectory(sc, idx, groups_bond_tensors(adj.groups, T), A, B, e, ALPHA, DT, nsteps)
    loss = ((eT - target.cpu()) ** 2).sum()
    loss.backward()
    assert abs(L_gpu - float(loss)) <= 1e-10 * abs(float(loss))
    assert np.allclose(g_gpu, theta.grad.numpy(), rtol=1e-8, atol=1e-12), (g_gpu, theta.grad.numpy())
    ge_ref = e.grad.numpy()
    assert np.abs(ge_gpu - ge_ref).max() <= 1e-8 * np.abs(ge_ref).max()


@pytest.mark.parametrize("precision", ["fp64", "fp64_fixed"])
def test_adjoint_matches_central_differences_128x128(cuda, precision):
    """The differentiable-LLG workload: 128 x 128 film, 2000 Heun steps, checkpoints every 100 steps;
    dL/d(J1, D, K, B_z) and three components of dL/de(0) against central differences, h = 1e-6, with
    the forward in either form."""
    from magex_gb300.adjoint import llg_trajectory
    nsteps = 2000
    sc, adj, S = _setup(128, nsteps, 100, precision)
    target = _target(adj, S, sc, nsteps)
    e0 = sc.init_spins("random", seed=1)
    theta0 = np.array([J1, D, K, BZ])
    _, g, ge = _loss_and_grads(adj, S, e0, target, theta0.tolist(), nsteps)

    def final(theta, e_init):
        T, A, B = _params(torch.as_tensor(theta, dtype=torch.float64), S)
        with torch.no_grad():
            return llg_trajectory(adj, torch.as_tensor(e_init, device=adj.device), T, A, B, nsteps)

    h = 1e-6
    for k in range(4):
        tp, tm = theta0.copy(), theta0.copy()
        tp[k] += h
        tm[k] -= h
        fd = _central_difference(final(tp, e0), final(tm, e0), target, h)
        assert abs(fd - g[k]) <= 1e-6 * max(abs(fd), 1e-3), (k, fd, g[k])
    for site, comp in [(0, 0), (4321, 2), (16000, 1)]:
        ep, em = e0.copy(), e0.copy()
        ep[site, comp] += h
        em[site, comp] -= h
        fd = _central_difference(final(theta0, ep), final(theta0, em), target, h)
        assert abs(fd - ge[site, comp]) <= 1e-6 * max(abs(fd), 1e-3), (site, comp, fd, ge[site, comp])


def test_adjoint_thermal_pathwise(cuda):
    """At T > 0 the gradient is the pathwise derivative of one Philox noise realisation: central
    differences with the same seed agree."""
    from magex_gb300.adjoint import AdjointLLG, llg_trajectory
    from magex_gb300.workloads import film_parameter_basis, triangular_film
    sc = triangular_film(L=24, field=(0, 0, BZ))
    adj = AdjointLLG(sc, alpha=ALPHA, dt=DT, temperature=15.0, seed=5, seg_steps=30)
    S = torch.as_tensor(group_basis(adj, film_parameter_basis(sc)), dtype=torch.float64)
    e0 = sc.init_spins("random", seed=3)
    target = torch.as_tensor(sc.init_spins("random", seed=4), device=adj.device)
    nsteps = 100
    _, g, _ = _loss_and_grads(adj, S, e0, target, [J1, D, K, BZ], nsteps)

    def final(theta):
        T, A, B = _params(torch.as_tensor(theta, dtype=torch.float64), S)
        with torch.no_grad():
            return llg_trajectory(adj, torch.as_tensor(e0, device=adj.device), T, A, B, nsteps)

    theta0 = np.array([J1, D, K, BZ])
    for k in range(4):
        tp, tm = theta0.copy(), theta0.copy()
        tp[k] += 1e-6
        tm[k] -= 1e-6
        fd = _central_difference(final(tp), final(tm), target, 1e-6)
        assert abs(fd - g[k]) <= 1e-6 * max(abs(fd), 1e-3), (k, fd, g[k])


def test_adjoint_shell_tensors_bcc(cuda):
    """Shell-tensor parameterisation of the two-site bcc model (4 shells, canonical and transposed
    bonds): d(mean energy after 40 steps)/dT_shell against central differences on sampled entries."""
    from magex_gb300.adjoint import AdjointLLG, CouplingGroups, llg_trajectory
    from magex_gb300.workloads import bcc_two_site, uniaxial_sia
    sc = bcc_two_site(L=4, J=(20.0, 10.0, -1.0, 1.0), dmi_frac=0.05, per="shell", seed=1, field=(0, 0, 0.3))
    groups = CouplingGroups.per_shell(sc)
    assert groups.ngroups == 4
    adj = AdjointLLG(sc, groups, alpha=0.05, dt=1e-4, seg_steps=16)
    T0 = torch.as_tensor(adj.T0)
    A0 = torch.as_tensor(np.stack([uniaxial_sia(0.01)] * 2))
    B0 = torch.tensor([0.0, 0.0, 0.3], dtype=torch.float64)
    e0 = torch.as_tensor(sc.init_spins("random", seed=7), device=adj.device)
    nsteps = 40
    N = sc.N

    def energy(e, T, A, B):
        from torch_reference import coupling_index
        idx = coupling_index(sc)
        Jb = groups_bond_tensors(groups, T).to(e.device)
        h = torch.zeros_like(e)
        for b, (src, dst) in enumerate(idx):
            h = h.index_add(0, src.to(e.device), e[dst.to(e.device)] @ Jb[b].T)
        As = A.to(e.device)[torch.as_tensor(sc.sublattice, device=e.device)]
        mu = torch.as_tensor(sc.mu, device=e.device)
        per_site = (torch.einsum("ia,iab,ib->i", e, As, e) - (e * h).sum(1)
                    - 5.7883818060e-2 * mu * (e @ B.to(e.device)))
        return per_site.sum() / N, per_site

    T = T0.clone().requires_grad_(True)
    eT = llg_trajectory(adj, e0, T, A0, B0, nsteps)
    loss, _ = energy(eT, T, A0, B0)
    loss.backward()
    g = T.grad.numpy()
    import math
    for (s, a, b) in [(0, 0, 0), (0, 1, 2), (1, 2, 1), (2, 0, 0), (3, 1, 0)]:
        vals = []
        for sgn in (1, -1):
            Tp = T0.clone()
            Tp[s, a, b] += sgn * 1e-6
            with torch.no_grad():
                ee = llg_trajectory(adj, e0, Tp, A0, B0, nsteps)
                _, per_site = energy(ee, Tp, A0, B0)
                vals.append(per_site.cpu().numpy())
        # exact summation of the per-site differences keeps the central difference free of rounding
        fd = math.fsum((vals[0] - vals[1]).tolist()) / N / 2e-6
        assert abs(fd - g[s, a, b]) <= 1e-6 * max(abs(fd), 1e-3), (s, a, b, fd, g[s, a, b])


def groups_bond_tensors(groups, T):
    Tb = T[torch.as_tensor(groups.group, dtype=torch.long)]
    tr = torch.as_tensor(groups.transposed, dtype=torch.bool)[:, None, None]
    return torch.where(tr, Tb.transpose(1, 2), Tb)


def test_adjoint_per_bond_groups_equal_pair_groups(cuda):
    """Per-coupling and reverse-pair parameterisations give the same gradient of the same loss."""
    from magex_gb300.adjoint import AdjointLLG, CouplingGroups, llg_trajectory
    from magex_gb300.workloads import film_parameter_basis, triangular_film, uniaxial_sia
    sc = triangular_film(L=20, field=(0, 0, BZ))
    S_bond = torch.as_tensor(film_parameter_basis(sc))
    e0 = torch.as_tensor(sc.init_spins("random", seed=1))
    target = torch.as_tensor(sc.init_spins("random", seed=2))
    grads = []
    for groups in (CouplingGroups.per_bond(sc), CouplingGroups.symmetric_pairs(sc)):
        adj = AdjointLLG(sc, groups, alpha=ALPHA, dt=DT, seg_steps=25)
        Sg = torch.zeros((groups.ngroups, 3, 3), dtype=torch.float64)
        for b in range(len(groups.group)):
            if not groups.transposed[b]:
                Sg[groups.group[b]] = S_bond[b]
        theta = torch.tensor([J1, D], dtype=torch.float64, requires_grad=True)
        T = theta[0] * torch.eye(3, dtype=torch.float64)[None] + theta[1] * Sg
        A = torch.as_tensor(uniaxial_sia(K))[None]
        B = torch.tensor([0.0, 0.0, BZ], dtype=torch.float64)
        eT = llg_trajectory(adj, e0.to(adj.device), T, A, B, 60)
        ((eT - target.to(adj.device)) ** 2).sum().backward()
        grads.append(theta.grad.numpy().copy())
    assert np.allclose(grads[0], grads[1], rtol=1e-10, atol=1e-12)


@pytest.mark.parametrize("precision", ["fp64", "fp64_fixed"])
def test_adjoint_resident_segments_equal_recompute(cuda, precision):
    """Keeping segments resident (no recomputation) gives the same gradient as recomputing them
    (bit for bit: the recomputation repeats the forward's arithmetic, in either form)."""
    from magex_gb300.adjoint import AdjointLLG, llg_trajectory
    from magex_gb300.workloads import film_parameter_basis, triangular_film, uniaxial_sia
    sc = triangular_film(L=24, field=(0, 0, BZ))
    e0 = torch.as_tensor(sc.init_spins("random", seed=1))
    target = torch.as_tensor(sc.init_spins("random", seed=2))
    out = []
    for cache in (0, 1 << 30, 3 * 8 * 14 * sc.N * 20):     # none, all, a part of the 5 segments
        adj = AdjointLLG(sc, alpha=ALPHA, dt=DT, seg_steps=20, cache_bytes=cache, precision=precision)
        S = torch.as_tensor(group_basis(adj, film_parameter_basis(sc)))
        theta = torch.tensor([J1, D], dtype=torch.float64, requires_grad=True)
        e = e0.clone().to(adj.device).requires_grad_(True)
        T = theta[0] * torch.eye(3, dtype=torch.float64)[None] + theta[1] * S
        A = torch.as_tensor(uniaxial_sia(K))[None]
        B = torch.tensor([0.0, 0.0, BZ], dtype=torch.float64)
        eT = llg_trajectory(adj, e, T, A, B, 100)
        ((eT - target.to(adj.device)) ** 2).sum().backward()
        out.append((theta.grad.numpy().copy(), e.grad.cpu().numpy()))
    for g, ge in out[1:]:
        assert np.array_equal(g, out[0][0]) and np.array_equal(ge, out[0][1])


@pytest.mark.parametrize("precision", ["fp64", "fp64_fixed"])
@pytest.mark.parametrize("precision_fwd", ["recompute", "resident"])
def test_adjoint_higher_onsite_terms_central_differences(cuda, golden_models, precision_fwd, precision):
    """Cubic (rotated axes) and higher uniaxial anisotropy in the adjoint: the spins' adjoint through
    the terms' Hessian and dL/dKc, dL/dK2, dL/dK3 (every site's constant moved together) against
    central differences (h = 1e-6) of the same trajectory, with segments recomputed or resident.
    Model: the sc system of the reference's sc_cubic fixture (Kc = 0.3, K2 = 0.2, K3 = 0.1 meV along
    [111], DMI, SIA) at T = 0 plus a triangular film with rotated cubic axes and K2 at 8 K."""
    from helpers import golden_supercell
    from magex_gb300.adjoint import AdjointLLG, llg_trajectory
    for tag, T_, nsteps in (("sc_cubic", 0.0, 60), ("tri_cubic_thermal", 8.0, 40)):
        sc, meta = golden_supercell(golden_models, tag)
        adj = AdjointLLG(sc, alpha=meta["alpha"], dt=meta["dt"], temperature=T_, seed=3, seg_steps=25,
                         cache_bytes=0 if precision_fwd == "recompute" else "auto", precision=precision)
        assert adj.has_higher
        T0 = torch.as_tensor(adj.T0)
        A0 = torch.as_tensor(np.asarray(sc.A_sub, float).reshape(sc.ns, 3, 3))
        B0 = torch.as_tensor(np.asarray(sc.B, float))
        H0 = adj.higher_params()
        e0 = sc.init_spins("random", seed=5)
        target = torch.as_tensor(sc.init_spins("random", seed=6), device=adj.device)
        H = torch.tensor(H0, dtype=torch.float64, requires_grad=True)
        e = torch.as_tensor(e0, device=adj.device).clone().requires_grad_(True)
        eT = llg_trajectory(adj, e, T0, A0, B0, nsteps, H=H)
        ((eT - target) ** 2).sum().backward()
        gH, ge = H.grad.numpy(), e.grad.cpu().numpy()

        def final(Hv, ev):
            with torch.no_grad():
                return llg_trajectory(adj, torch.as_tensor(ev, device=adj.device), T0, A0, B0, nsteps,
                                      H=torch.as_tensor(Hv, dtype=torch.float64))

        h = 1e-6
        present = [sc.cubic is not None] + [sc.uniaxial_higher is not None] * 2
        for k in range(3):
            if not present[k]:
                assert gH[k] == 0.0
                continue
            Hp, Hm = H0.copy(), H0.copy()
            Hp[k] += h
            Hm[k] -= h
            fd = _central_difference(final(Hp, e0), final(Hm, e0), target, h)
            assert abs(fd - gH[k]) <= 1e-6 * max(abs(fd), 1e-3), (tag, k, fd, gH[k])
        for site, comp in [(0, 0), (7, 2), (sc.N - 1, 1)]:
            ep, em = e0.copy(), e0.copy()
            ep[site, comp] += h
            em[site, comp] -= h
            fd = _central_difference(final(H0, ep), final(H0, em), target, h)
            assert abs(fd - ge[site, comp]) <= 1e-6 * max(abs(fd), 1e-3), (tag, site, comp, fd, ge[site, comp])


def test_adjoint_accumulates_only_requested_gradients(cuda):
    """autograd asks the adjoint only for the inputs that require grad (mgx_adjoint_set_needs): the
    coupling gradient alone equals, bit for bit, the one computed together with the single-ion and
    field gradients, and the spins' adjoint is unchanged."""
    from magex_gb300.adjoint import llg_trajectory
    sc, adj, S = _setup(24, 60, 20)
    e0 = sc.init_spins("random", seed=1)
    target = torch.as_tensor(sc.init_spins("random", seed=2), device=adj.device)
    out = []
    for all_params in (True, False):
        theta = torch.tensor([J1, D, K, BZ], dtype=torch.float64, requires_grad=True)
        T, A, B = _params(theta, S)
        if not all_params:
            A, B = A.detach(), B.detach()
        e = torch.as_tensor(e0, device=adj.device).clone().requires_grad_(True)
        ((llg_trajectory(adj, e, T, A, B, 60) - target) ** 2).sum().backward()
        out.append((theta.grad.numpy().copy(), e.grad.cpu().numpy()))
    assert np.array_equal(out[0][0][:2], out[1][0][:2])        # dL/dJ1, dL/dD through T
    assert np.all(out[1][0][2:] == 0.0) and np.all(out[0][0][2:] != 0.0)
    assert np.array_equal(out[0][1], out[1][1])


def test_fixed_point_adjoint_equals_fp64_adjoint(cuda):
    """The adjoint with the forward and the transposed gathers in exact 56-bit fixed point (the
    neighbours' g in block floating point, aligned to the largest exponent) gives the gradients of
    the all-FP64 adjoint to rounding: two-site bcc with four shells of full per-shell tensors (50
    couplings per site), 300 K, d(mean energy after 30 steps)/d(shell tensors) and d/de(0)."""
    from magex_gb300.adjoint import AdjointLLG, CouplingGroups, energy_per_site, llg_trajectory
    from magex_gb300.workloads import bcc_two_site, uniaxial_sia
    sc = bcc_two_site(L=6, J=(20.0, 10.0, -1.0, 1.0), dmi_frac=0.05, per="shell", seed=1, field=(0, 0, 0.3))
    groups = CouplingGroups.per_shell(sc)
    A0 = torch.as_tensor(np.stack([uniaxial_sia(0.01)] * 2))
    B0 = torch.tensor([0.0, 0.0, 0.3], dtype=torch.float64)
    out = {}
    for precision in ("fp64", "fp64_fixed"):
        adj = AdjointLLG(sc, groups, alpha=0.05, dt=1e-4, temperature=300.0, seed=4, seg_steps=10,
                         cache_bytes=0, precision=precision)
        T = torch.as_tensor(adj.T0).clone().requires_grad_(True)
        e = torch.as_tensor(sc.init_spins("random", seed=7), device=adj.device).requires_grad_(True)
        eT = llg_trajectory(adj, e, T, A0, B0, 30)
        energy_per_site(sc, groups, eT, T, A0, B0).mean().backward()
        out[precision] = (T.grad.numpy().copy(), e.grad.cpu().numpy())
    gT64, ge64 = out["fp64"]
    gTfx, gefx = out["fp64_fixed"]
    assert np.abs(gTfx - gT64).max() <= 1e-10 * np.abs(gT64).max()
    assert np.abs(gefx - ge64).max() <= 1e-10 * np.abs(ge64).max()
