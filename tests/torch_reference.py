"""Dense FP64 PyTorch restatement of the Heun step, for checking the adjoint with torch autograd.

TEST INFRASTRUCTURE ONLY.  The step is magex/llg.py:216-227 with the field of
magex/spinmodel.py:454-473 written with index_add over the stencil couplings, so that torch autograd
differentiates it with respect to the spins and every coupling tensor.
"""
import numpy as np
import torch

from magex_gb300.constants import GAMMA, MU_B


def coupling_index(sc):
    """Per stencil coupling b: (src, dst) site indices (magex order) of every cell where it acts."""
    L = np.array(sc.L)
    c = np.stack(np.meshgrid(*[np.arange(n) for n in sc.L], indexing="ij"), -1).reshape(-1, 3)
    cidx = lambda q: (q[:, 0] * L[1] + q[:, 1]) * L[2] + q[:, 2]      # noqa: E731
    out = []
    for b in range(len(sc.bond_src)):
        t = c + sc.bond_R[b][None, :]
        ok = np.ones(len(c), bool)
        for a in range(3):
            if sc.pbc[a]:
                t[:, a] %= L[a]
            else:
                ok &= (t[:, a] >= 0) & (t[:, a] < L[a])
        src = cidx(c[ok]) * sc.ns + sc.bond_src[b]
        dst = cidx(t[ok]) * sc.ns + sc.bond_dst[b]
        out.append((torch.as_tensor(src), torch.as_tensor(dst)))
    return out


def heun_trajectory(sc, index, Jb, A, B, e0, alpha, dt, nsteps, precession=True):
    """e after nsteps T = 0 Heun steps; Jb (nbond,3,3), A (ns,3,3), B (3) and e0 (N,3) torch fp64."""
    mu = torch.as_tensor(sc.mu, dtype=torch.float64)
    inv = 1.0 / (mu * MU_B)
    sub = torch.as_tensor(sc.sublattice)
    As = A[sub]
    pre = -GAMMA / (1.0 + alpha * alpha)

    def field(e):
        h = torch.zeros_like(e)
        for b, (src, dst) in enumerate(index):
            h = h.index_add(0, src, e[dst] @ Jb[b].T)
        Ae = torch.einsum("iab,ib->ia", As, e)
        return (2.0 * h - 2.0 * Ae) * inv[:, None] + B[None, :]

    def rhs(e, H):
        c = torch.cross(e, H, dim=1)
        d = torch.cross(e, c, dim=1)
        return pre * (c + alpha * d) if precession else pre * alpha * d

    def unit(v):
        return v / torch.linalg.vector_norm(v, dim=1, keepdim=True)

    e = e0
    for _ in range(nsteps):
        k1 = rhs(e, field(e))
        ep = unit(e + dt * k1)
        k2 = rhs(ep, field(ep))
        e = unit(e + 0.5 * dt * (k1 + k2))
    return e
