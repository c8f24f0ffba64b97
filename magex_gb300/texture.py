"""Topological charge of one atomic layer (magex/texture.py:14-63), evaluated on the GB300.

magex triangulates the layer with a periodic Delaunay construction (3 x 3 tiling, triangles whose
centroid lies in the central supercell) and sums the Berg-Luscher solid angles on every call; the
triangulation alone takes seconds at 10^5 spins.  Here the same triangles are built once per
(system, plane, layer) on the host (scipy, the same construction and orientation signs), kept, and
every call sums the solid angles of the current spins on the device (``mgx_topological_charge``).
"""
from __future__ import annotations

import numpy as np
import torch

from .device import DeviceModel, supercell_from_system

PLANES = {"xy": (0, 1, 2), "xz": (0, 2, 1), "yz": (1, 2, 0)}

CACHE_SIZE = 8
_cache = {}


def layer_indices(system, plane="xy", layer=0, tol=0.05):
    """Indices of the spins in one atomic layer normal to the plane; layer may be negative
    (magex/texture.py:14-20)."""
    a, b, n = PLANES[plane]
    z = np.asarray(system.positions)[:, n]
    levels = np.unique(np.round(z / tol) * tol)
    lev = levels[layer]
    return np.where(np.abs(z - lev) < tol * 1.01)[0], (a, b, n), len(levels)


def _inplane_supercell_vectors(system, axes):
    a, b, n = axes
    V = np.array(system.L)[:, None] * system.uc.cell
    order = np.argsort(np.abs(V[:, n]))
    return V[order[:2]][:, [a, b]], [bool(system.pbc[k]) for k in order[:2]]


def layer_triangles(system, plane="xy", layer=0):
    """(T, 3) site indices and (T,) signs (orientation times the handedness of the plane's axes) of
    magex's periodic Delaunay triangulation of a layer, or None when magex's charge is 0 by
    construction (fewer than 3 spins, or no triangulation)."""
    from scipy.spatial import Delaunay
    idx, axes, _ = layer_indices(system, plane, layer)
    if len(idx) < 3:
        return None
    a, b, n = axes
    P = np.asarray(system.positions)[idx][:, [a, b]]
    V, per = _inplane_supercell_vectors(system, axes)
    shifts = [(i, j) for i in ((-1, 0, 1) if per[0] else (0,)) for j in ((-1, 0, 1) if per[1] else (0,))]
    Pt = np.concatenate([P + i * V[0] + j * V[1] for i, j in shifts])
    try:
        tri = Delaunay(Pt).simplices
    except Exception:
        return None
    cen = Pt[tri].mean(1)
    frac = np.linalg.solve(V.T, (cen - 0.0).T).T
    keep = np.all((frac >= -1e-9) & (frac < 1 - 1e-9), axis=1) if len(shifts) > 1 else np.ones(len(tri), bool)
    tri = tri[keep]
    p1, p2, p3 = Pt[tri[:, 0]], Pt[tri[:, 1]], Pt[tri[:, 2]]
    orient = np.sign((p2[:, 0] - p1[:, 0]) * (p3[:, 1] - p1[:, 1]) - (p2[:, 1] - p1[:, 1]) * (p3[:, 0] - p1[:, 0]))
    hand = 1.0 if plane in ("xy", "yz") else -1.0
    return idx[tri % len(idx)], hand * orient


def topological_charge(system, e, plane="xy", layer=0):
    """Skyrmion number Q = (1/4 pi) sum of the triangles' solid angles (magex/texture.py:30-63) of
    spins e ((N, 3) numpy array or torch tensor, magex order).  The triangulation and the device copy
    of the model are kept for the next calls on the same system, plane and layer (the last
    ``CACHE_SIZE`` of them)."""
    key = (id(system), plane, layer, system.N, tuple(system.L))
    hit = _cache.pop(key, None)
    if hit is None:
        tris = layer_triangles(system, plane, layer)
        dm = None
        if tris is not None and len(tris[0]):
            dm = DeviceModel(supercell_from_system(system))
            dm.set_triangles(*tris)
        hit = (system, dm)                        # the system is held so that its id stays unique
    _cache[key] = hit
    while len(_cache) > CACHE_SIZE:
        _cache.pop(next(iter(_cache)))
    dm = hit[1]
    if dm is None:
        return 0.0
    return float(dm.topological_charge(dm.to_lattice(e)).item())
