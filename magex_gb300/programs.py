"""Ferromagnetic-resonance ring-down (magex/programs.py:124-150, ``fmr``) on the GB300.

magex relaxes the spins, then integrates the LLG equation after a short in-plane field step
(``field_func`` on for t < 5 dt), recording the mean spin every ``every`` steps, and takes the
resonance from the Hann-windowed spectrum of the component along the pulse, refined by a parabola
through the logarithm of the three bins around the peak.  Here the steps run on the device: the
pulse steps go through the solver's field hook, the free ring-down as graph replays between samples,
and each sample is one device reduction into a device buffer that is read once at the end.

The relaxation is the damped-LLG ``minimize(..., "llg", tol=1e-7)`` of this package; magex uses
its host L-BFGS there.  From a relaxed state both return at once, and the ring-downs agree.
"""
from __future__ import annotations

import numpy as np
import torch

from .llg import GB300LLG
from .minimize import minimize


def _peak_frequency(f, F):
    """Frequency of the largest non-DC bin, refined by a parabola through log F at the peak and its
    two neighbours (interpolated on the bin index)."""
    k = int(np.argmax(F[1:]) + 1)
    x = float(k)
    if 1 <= k < len(F) - 1:
        lm, l0, lp = np.log(F[k - 1:k + 2] + 1e-300)
        x = k + 0.5 * (lm - lp) / (lm - 2 * l0 + lp)
    return float(np.interp(x, np.arange(len(f)), f))


def fmr(system, e, B_pulse=0.01, direction=(1, 0, 0), alpha=0.001, dt=2e-3, steps=20000, every=5, log=None,
        integrator="heun"):
    """Ring-down after a field step of B_pulse (T) along ``direction`` lasting 5 dt; returns
    ((f GHz, |FFT|), f_peak GHz, table (t, <e>)) as magex/programs.py:124-150."""
    e, _ = minimize(system, e, "llg", tol=1e-7)
    p = np.asarray(direction, float)
    p = p / np.linalg.norm(p)
    sol = GB300LLG(system, alpha, dt, 0.0, integrator=integrator)
    t0 = 5 * dt
    sol.field_func = lambda t: (B_pulse * p if t < t0 else np.zeros(3))
    dm = sol.model
    N = sol.sc.N
    lat = dm.to_lattice(e)
    steps, every = int(steps), int(every)
    sums = torch.empty((len(range(0, steps, every)), 8), dtype=torch.float64, device=dm.device)
    ts = []

    def record():
        sums[len(ts)].copy_(dm.observables(lat))
        ts.append(sol.time)

    n = 0
    while n < steps and sol.time < t0:          # a stage of this step still sees the pulse
        sol.step_lattice(lat)
        if n % every == 0:
            record()
        n += 1
    sol.field_func = None                       # field_func is zero from here on
    while n < steps:
        m = n + (-n) % every                    # the next step after which magex samples
        if m >= steps:
            sol.run_lattice(lat, steps - n)
            break
        sol.run_lattice(lat, m - n + 1)
        record()
        n = m + 1
    ms = sums[:len(ts), 1:4].cpu().numpy() / N
    c = int(np.argmax(np.abs(p)))
    sig = (ms[:, c] - ms[:, c].mean()) * np.hanning(len(ms))
    F = np.abs(np.fft.rfft(sig))
    f = np.fft.rfftfreq(len(sig), d=every * dt) * 1e3       # dt in ps: GHz
    fpk = _peak_frequency(f, F)
    if log:
        log(f"  FMR peak at {fpk:.3f} GHz")
    return (f, F), fpk, np.column_stack([ts, ms])
