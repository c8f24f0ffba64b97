"""S(q, w) sampling with the spins kept on the GB300 (magex/spectra.py:49-84, structure_factor).

magex multiplies a dense (N, nq) phase matrix into the spins on the host at every sample, so at
10^6 spins the sampling, not the LLG step, dominates and every sample crosses PCIe.  Here the LLG
steps run on the device (``GB300LLG.run_lattice``), the projection m_q is a two-stage separable
Fourier kernel (``mgx_fourier_project``) writing into a device buffer, the order vector is summed
on the device, and only the (nsamp, nq, 3) samples come back for magex's Welch / Hann averaging.
"""
from __future__ import annotations

import ctypes as C
import time

import numpy as np
import torch

from . import _lib
from .constants import HBAR_MEV_PS
from .device import stream_ptr
from .lattice import NeighbourList


class FourierProjector:
    """m_q = N^-1/2 sum_i e_i exp(-i q.r_i) of device spins for fractional wave vectors qfrac (nq, 3)
    of the unit cell's reciprocal lattice (reciprocal vectors 2 pi inv(cell)^T, magex/spectra.py:53)."""

    def __init__(self, model, qfrac):
        sc = model.sc
        if isinstance(sc, NeighbourList):
            raise NotImplementedError("the separable Fourier projection needs a lattice (Supercell) model")
        self.model = model
        self.lib = _lib.load()
        qf = np.ascontiguousarray(np.asarray(qfrac, float).reshape(-1, 3))
        self.nq = len(qf)
        cell = np.asarray(sc.uc.cell, float)
        B = 2 * np.pi * np.linalg.inv(cell).T
        qc = qf @ B
        pos = np.asarray(sc.uc.positions, float).reshape(sc.ns, 3)
        ph = np.exp(-1j * (pos @ qc.T)).T                       # (nq, ns)
        sub = np.ascontiguousarray(np.stack([ph.real, ph.imag], -1).reshape(-1))
        h = C.c_void_p()
        _lib.check(self.lib.mgx_fourier_create(model.handle, self.nq, _lib.dptr(qf), _lib.dptr(sub), C.byref(h)),
                   "mgx_fourier_create")
        self.handle = h

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            try:
                self.lib.mgx_fourier_destroy(h)
            except Exception:
                pass
            self.handle = None

    def project(self, lat, out=None, stream=None):
        """(nq, 3) complex128 device tensor m_q of lattice-layout spins lat."""
        out = torch.empty((self.nq, 3), dtype=torch.complex128, device=lat.device) if out is None else out
        _lib.check(self.lib.mgx_fourier_project(self.handle, C.c_void_p(lat.data_ptr()), C.c_void_p(out.data_ptr()),
                                                stream_ptr(stream)), "mgx_fourier_project")
        return out


def _frame(n):
    n = np.asarray(n, float) / np.linalg.norm(n)
    a = np.array([1.0, 0, 0]) if abs(n[0]) < 0.9 else np.array([0, 1.0, 0])
    e1 = np.cross(n, a)
    e1 /= np.linalg.norm(e1)
    return e1, np.cross(n, e1), n


def structure_factor(system, solver, e, qfrac, nsteps, sample_every=10, nseg=4, log=None):
    """Drop-in for magex.spectra.structure_factor with a GB300LLG solver: runs nsteps LLG steps,
    samples m_q every sample_every steps on the device, and returns (E_meV, S_perp, S_par, e) with
    magex's transverse / longitudinal split about the mean order vector and its Hann-windowed Welch
    average over nseg segments."""
    model = solver.model
    proj = FourierProjector(model, qfrac)
    lat = model.to_lattice(e)
    nsamp = nsteps // sample_every
    mq = torch.empty((nsamp, proj.nq, 3), dtype=torch.complex128, device=lat.device)
    ref = torch.zeros(3, dtype=torch.float64, device=lat.device)
    t0 = time.time()
    for s in range(nsamp):
        solver.run_lattice(lat, sample_every)
        ref += model.observables(lat)[4:7]
        proj.project(lat, out=mq[s])
    mq = mq.cpu().numpy()
    e1, e2, n = _frame(ref.cpu().numpy())
    dt = solver.dt * sample_every
    seg = nsamp // nseg
    win = np.hanning(seg)
    Sperp = 0.0
    Spar = 0.0
    for k in range(nseg):
        x = mq[k * seg:(k + 1) * seg]
        x = x - x.mean(0, keepdims=True)
        F = np.fft.fft(x * win[:, None, None], axis=0)
        Sperp = Sperp + np.abs(F @ e1) ** 2 + np.abs(F @ e2) ** 2
        Spar = Spar + np.abs(F @ n) ** 2
    f = np.fft.fftfreq(seg, dt)
    E = 2 * np.pi * f * HBAR_MEV_PS
    order = np.argsort(E)
    if log:
        log(f"  S(q,w): {nsamp} samples x {proj.nq} q-points, {nseg} segments, dE = {E[1] - E[0]:.3f} meV, "
            f"E_max = {E.max():.1f} meV, {time.time() - t0:.1f} s")
    e_out = model.from_lattice(lat).cpu().numpy()
    return E[order], (Sperp / nseg)[order].T, (Spar / nseg)[order].T, e_out
