"""Damped-LLG relaxation (magex/minimize.py:168-179, ``minimize(system, e, "llg", ...)``) on the GB300.

magex relaxes with its own LLG solver at alpha = 1, dt = 2 fs, T = 0 and no precession, checking
the largest torque every 50 steps (in meV: |e x B_eff|_max mu_B max(mu) < tol).  Here the spins stay
on the device: 50 steps are one replay of a step graph and each check is one reduction
(``mgx_observables``) whose result is read while the next 50 steps run.

The other methods of magex's dispatcher (L-BFGS, NCG, velocity projection) are host optimisers that
do not use the LLG step; they raise NotImplementedError.
"""
from __future__ import annotations

import numpy as np
import torch

from .constants import MU_B
from .llg import GB300LLG

HOST_METHODS = ("lbfgs", "lbfgs_oso", "ncg", "vp")
CHECK_EVERY = 50


def minimize(system, e, method="llg", tol=1e-6, max_iter=None, log=None):
    """Relax spins e ((N, 3), magex order) of ``system``; returns (e, {"iterations", "energy"}) as
    magex/minimize.py:168-181.  ``iterations`` is the index of the torque check that stopped the loop
    (max_iter - 1 when none did), ``energy`` the total energy (meV) of the returned spins."""
    if method in HOST_METHODS:
        raise NotImplementedError(f"minimiser '{method}' is a host optimiser, not the LLG path; use method='llg'")
    if method != "llg":
        raise ValueError(f"unknown minimiser '{method}'")
    sol = GB300LLG(system, 1.0, 2e-3, 0.0, precession=False)
    dm = sol.model
    lat = dm.to_lattice(np.asarray(e, float))
    at_check = torch.empty_like(lat)
    torque = torch.empty(1, dtype=torch.float64, pin_memory=True)
    ready = torch.cuda.Event()
    scale = MU_B * float(np.max(sol.sc.mu))
    n = int(max_iter or 100000)
    k, stopped = 0, False
    while k < n:
        # the check of the spins at step k travels to the host while the next steps already run
        # (T = 0: no noise, so steps past a passing check change nothing but the discarded spins)
        torque.copy_(dm.observables(lat)[7:8], non_blocking=True)
        ready.record()
        at_check.copy_(lat)
        m = min(CHECK_EVERY, n - k)
        sol.run_lattice(lat, m)
        ready.synchronize()
        if float(torque[0]) * scale < tol:
            lat, stopped = at_check, True
            break
        k += m
    it = k if stopped else n - 1
    E = float(dm.observables(lat)[0].item())
    out = dm.from_lattice(lat).cpu().numpy()
    pinned = getattr(system, "pinned", None)
    if pinned is not None and not callable(system):
        out[pinned] = system.pinned_dir[pinned]
    if log:
        log(f"  LLG relaxation: {it} iterations, E = {E:.6f} meV")
    return out, dict(iterations=it, energy=E)
