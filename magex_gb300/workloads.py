"""Synthetic spin models of the benchmark workloads (seeded, no external data).

  sc_model            simple cubic, isotropic nearest-neighbour J (magex benchmarks/sc.json shape)
  bcc_two_site_model  bcc metal in its two-site cubic cell with per-bond (or per-shell) full 3x3
                      tensors: isotropic shells + random symmetric traceless part + random DMI,
                      J_ji = J_ij^T for every reverse bond, uniaxial SIA, written as a results.json
                      dict (magex's own "bcc" lattice is the one-site primitive cell,
                      magex/models.py:30, so the two-site cell is built here)
  triangular_film     triangular monolayer with interfacial DMI and SIA (magex make_model)
  film_ensemble       seeded parameters of an ensemble of uneven triangular films
"""
from __future__ import annotations

import itertools

import numpy as np

from .lattice import Supercell
from .spinmodel import load_results, make_model, skew


def sc_model(J=1.0, moment=2.0, a=3.0, **kw):
    return make_model("sc", a=a, J=[J], moment=moment, **kw)


def _random_sym_traceless(rng, norm):
    X = rng.normal(size=(3, 3))
    S = 0.5 * (X + X.T)
    S -= np.trace(S) / 3 * np.eye(3)
    return S * (norm / np.linalg.norm(S))


def _random_unit(rng):
    v = rng.normal(size=3)
    return v / np.linalg.norm(v)


def bcc_two_site_model(J=(20.0, 10.0, -1.0), a=2.87, aniso=0.01, dmi=1.0, dmi_frac=None, K=0.01,
                       moment=2.2, seed=0, per="bond"):
    """results.json dict of two-site cubic bcc with len(J) shells (8, 6, 12, 24, ... neighbours).

    Every unordered bond {(i, j, R), (j, i, -R)} gets one tensor J_iso I + S + skew(D) on its
    canonical orientation (i < j, or i == j and R > 0 lexicographically) and the transpose on the
    reverse one, so h_i = sum_j J_ij e_j is the exact gradient.  S is symmetric traceless with
    Frobenius norm aniso * |J_iso|; |D| = dmi (meV), or dmi_frac * |J_iso| when dmi_frac is given.
    per="bond" draws (S, D) for every canonical bond of the cell, per="shell" once per shell.
    """
    rng = np.random.default_rng(seed)
    cell = a * np.eye(3)
    frac = np.array([[0, 0, 0], [0.5, 0.5, 0.5]])
    pos = frac @ cell
    cand = []
    span = range(-3, 4)
    for i, j in itertools.product(range(2), repeat=2):
        for R in itertools.product(span, repeat=3):
            if i == j and R == (0, 0, 0):
                continue
            r = pos[j] + np.array(R) @ cell - pos[i]
            cand.append((round(float(np.linalg.norm(r)), 6), i, j, R))
    dists = sorted({c[0] for c in cand})[:len(J)]
    shell_of = {d: k for k, d in enumerate(dists)}
    cand = [c for c in cand if c[0] in shell_of]
    shell_draw = {}
    tensors = {}
    for d, i, j, R in cand:
        canonical = i < j or (i == j and R > (0, 0, 0))
        if not canonical:
            continue
        sh = shell_of[d]
        Jiso = float(J[sh])
        if per == "shell":
            if sh not in shell_draw:
                shell_draw[sh] = (_random_sym_traceless(rng, aniso * abs(Jiso)), _random_unit(rng))
            S, u = shell_draw[sh]
        else:
            S, u = _random_sym_traceless(rng, aniso * abs(Jiso)), _random_unit(rng)
        Dmag = dmi if dmi_frac is None else dmi_frac * abs(Jiso)
        T = Jiso * np.eye(3) + S + skew(Dmag * u)
        tensors[(i, j, R)] = T
        tensors[(j, i, tuple(-x for x in R))] = T.T
    mesh = [64, 64, 64]
    pairs = []
    for d, i, j, R in cand:
        T = tensors[(i, j, R)]
        pairs.append(dict(i=i, j=j, R=list(R), nu=[int(R[k]) % mesh[k] for k in range(3)], dist=d,
                          vec=(pos[j] + np.array(R) @ cell - pos[i]).tolist(), J=T.tolist(), resid=0.0,
                          degeneracy=1))
    z = np.array([0.0, 0.0, 1.0])
    A_ion = -K * (np.outer(z, z) - np.eye(3) / 3)
    return dict(version="model", sites=[0, 1], symbols=["Fe", "Fe"], cell=cell.tolist(), positions=pos.tolist(),
                mesh=mesh, moments=[(moment * z).tolist()] * 2, charges=[0.0, 0.0], refs=[z.tolist()],
                full_tensor=True, A=[A_ion.tolist()] * 2, mu=0.0, mag_pos=[0, 1], lig_pos=[], pairs=pairs,
                corrections={}, lloyd=None, mae=None, symmetry=None, four_spin=None,
                model=dict(lattice="bcc-two-site", a=a, J=list(J), aniso=aniso, dmi=dmi, K=K, moment=moment,
                           seed=seed, per=per))


def bcc_two_site(L=128, field=(0.0, 0.0, 0.5), **kw):
    """Supercell L^3 of the two-site bcc model (N = 2 L^3)."""
    return Supercell(load_results(bcc_two_site_model(**kw)), (L, L, L), (True, True, True), field)


def triangular_film_model(J=1.0, D=0.3, K=0.05, moment=2.0, a=3.0):
    return make_model("triangular", a=a, J=[J], D=D, dmi="interfacial", K=K, moment=moment)


def triangular_film(L=128, field=(0.0, 0.0, 2.0), **kw):
    return Supercell(load_results(triangular_film_model(**kw)), (L, L, 1), (True, True, False), field)


def film_ensemble(n=256, sides=tuple(range(32, 257, 16)), Bmax=3.0, Tmax=20.0, seed=0):
    """Seeded (L, B_z, T) of an ensemble of uneven triangular films."""
    rng = np.random.default_rng(seed)
    L = rng.choice(np.array(sides), size=n)
    Bz = rng.uniform(0.0, Bmax, size=n)
    T = rng.uniform(0.0, Tmax, size=n)
    return [dict(L=int(L[k]), B=(0.0, 0.0, float(Bz[k])), T=float(T[k])) for k in range(n)]


def triangle_list(sc):
    """Two triangles per cell of a periodic triangular monolayer (magex site order) with orientation
    +1: (c, c+a1, c+a2) and (c+a1, c+a1+a2, c+a2).  On a perfect triangular lattice this is the
    periodic Delaunay triangulation that magex/texture.py:30-63 builds, so the Berg-Luscher sums
    agree."""
    L0, L1, _ = sc.L
    if sc.ns != 1 or sc.L[2] != 1:
        raise ValueError("triangle_list expects a one-site monolayer (L, L, 1)")
    i, j = np.meshgrid(np.arange(L0), np.arange(L1), indexing="ij")
    idx = lambda a, b: ((a % L0) * L1 + (b % L1))       # noqa: E731
    t1 = np.stack([idx(i, j), idx(i + 1, j), idx(i, j + 1)], -1).reshape(-1, 3)
    t2 = np.stack([idx(i + 1, j), idx(i + 1, j + 1), idx(i, j + 1)], -1).reshape(-1, 3)
    tri = np.concatenate([t1, t2])
    return tri, np.ones(len(tri))


def film_parameter_basis(sc, normal=(0.0, 0.0, 1.0)):
    """For a one-shell film with interfacial DMI (make_model "triangular"/"square" with D): the constant
    matrices S_b = skew(n x r_b / |r_b|) of every stencil coupling, so that J_b = J1 I + D S_b (exact
    for the couplings make_model writes).  Returns (S (nbond, 3, 3))."""
    uc = sc.uc
    n = np.asarray(normal, float) / np.linalg.norm(normal)
    S = []
    for i, j, R in zip(sc.bond_src, sc.bond_dst, sc.bond_R):
        r = uc.positions[j] + R @ uc.cell - uc.positions[i]
        S.append(skew(np.cross(n, r / np.linalg.norm(r))))
    return np.array(S)


def uniaxial_sia(K, axis=(0.0, 0.0, 1.0)):
    """Traceless single-ion tensor -K (n n^T - I/3) of magex/models.py:109."""
    n = np.asarray(axis, float) / np.linalg.norm(axis)
    return -K * (np.outer(n, n) - np.eye(3) / 3)
