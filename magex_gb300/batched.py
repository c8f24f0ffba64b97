"""Batched ensemble of independent LLG systems on one GB300.

    ens = BatchedLLG([film(L) for L in sides], alpha=0.1, dt=1e-4, temperature=Ts, seed=seeds)
    ens.set_spins([sc.init_spins("random", seed=k) for k, sc in enumerate(ens.systems)])
    ens.autotune()
    ens.run(5000)                               # one persistent launch per stage, CUDA-graph replays
    E = ens.observables()[:, 0]                 # per-system energy (meV)
    Q = ens.topological_charge()                # per-system skyrmion number

magex steps each system with its own ``LLGSolver`` (``magex/llg.py:216-227``); an ensemble of
replicas, temperatures, fields or lattices is a Python loop over solvers.  Here all systems share
one device spin array (system k is the (3, N_k) lattice-layout block at 3*offset_k) and every stage
is one launch over a tile list (libmgx ``mgx_batch_*``).  Each system keeps its own stencil, field,
damping, temperature and Philox key, so system k evolves exactly as ``GB300LLG`` would evolve it
alone with the same seed.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib
from .constants import GAMMA, K_B, MU_B
from .device import DeviceModel, stream_ptr, supercell_from_system
from .llg import AUTO_FIXED_MIN_SITES, _SUPPORTED, _philox_key, fixed_point_eligible


def _per_system(x, n, name):
    if np.isscalar(x) or x is None:
        return [x] * n
    x = list(x)
    if len(x) != n:
        raise ValueError(f"{name} must be a scalar or have one entry per system ({n})")
    return x


class BatchedLLG:
    """An ensemble of independent Heun / Depondt LLG systems stepped by shared launches."""

    def __init__(self, systems, alpha=0.1, dt=1e-3, temperature=0.0, seed=None, precession=True,
                 integrator="heun", noise="philox", precision="auto", device=None):
        if integrator not in _SUPPORTED:
            raise NotImplementedError(f"integrator '{integrator}' is not implemented by the GB300 kernels")
        if noise not in ("philox", "host"):
            raise ValueError("noise must be 'philox' or 'host'")
        if precision not in ("fp64", "fp64_fixed", "auto"):
            raise ValueError("batched systems use precision 'auto', 'fp64' or 'fp64_fixed'")
        self.systems = [supercell_from_system(s) for s in systems]
        if precision == "auto":
            # the exact fixed-point sum form when every system supports it, the ensemble holds at least
            # AUTO_FIXED_MIN_SITES sites and some system has couplings beyond isotropic numbers (the
            # per-system choice of GB300LLG's "auto" made for the whole launch)
            alphas = _per_system(alpha, len(self.systems), "alpha")
            ok = all(fixed_point_eligible(sc, a) for sc, a in zip(self.systems, alphas))
            ok = ok and sum(sc.N for sc in self.systems) >= AUTO_FIXED_MIN_SITES
            ok = ok and any(int(sc.width) != 1 for sc in self.systems)
            precision = "fp64_fixed" if ok else "fp64"
        self.precision = precision
        n = len(self.systems)
        if n == 0:
            raise ValueError("empty ensemble")
        for sc in self.systems:
            if sc.alpha_site is not None or sc.site_T is not None or sc.mu_site is not None:
                raise NotImplementedError("batched systems take uniform damping, temperature and moments per sublattice")
        self.nsys = n
        self.models = [DeviceModel(sc, device) for sc in self.systems]
        self.device = self.models[0].device
        self.lib = self.models[0].lib
        self.alpha = [float(a) for a in _per_system(alpha, n, "alpha")]
        self.dt = [float(d) for d in _per_system(dt, n, "dt")]
        self.T = [float(t) for t in _per_system(temperature, n, "temperature")]
        seeds = _per_system(seed, n, "seed")
        self.seeds = seeds
        self.noise = noise
        self.integrator = integrator
        params = (_lib.LLGParams * n)()
        for k in range(n):
            p = params[k]
            p.dt = self.dt[k]
            p.alpha = self.alpha[k]
            p.alpha_site = None
            p.precession = int(bool(precession))
            p.integrator = _SUPPORTED[integrator]
            p.noise = _lib.NOISE_HOST if noise == "host" else _lib.NOISE_PHILOX
            p.seed = _philox_key(seeds[k])
            p.precision = _lib.PRECISION_FP64_FIXED_GATHER if precision == "fp64_fixed" else _lib.PRECISION_FP64
        handles = (C.c_void_p * n)(*[m.handle.value for m in self.models])
        h = C.c_void_p()
        with torch.cuda.device(self.device):
            _lib.check(self.lib.mgx_batch_create(handles, params, n, C.byref(h)), "mgx_batch_create")
        self.handle = h
        self.offsets = np.array([self.lib.mgx_batch_offset(h, k) for k in range(n + 1)], np.int64)
        self.ntot = int(self.offsets[-1])
        self.e = torch.zeros(3 * self.ntot, dtype=torch.float64, device=self.device)
        self._obs = torch.empty((n, 8), dtype=torch.float64, device=self.device)
        self._Q = torch.empty(n, dtype=torch.float64, device=self.device)
        self._noise = None
        self._rngs = [np.random.default_rng(s) for s in seeds] if noise == "host" else None
        self.time = 0.0
        self._step_index = 0
        self.launch = (256, 0)
        for k in range(n):
            self._push_sigma(k)

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            try:
                self.lib.mgx_batch_destroy(h)
            except Exception:
                pass
            self.handle = None

    # ------------------------------------------------------------------ parameters
    def _push_sigma(self, k):
        sc = self.systems[k]
        if self.T[k] > 0:
            sig = np.sqrt(2.0 * self.alpha[k] * K_B * self.T[k] / (GAMMA * sc.mu_sub * MU_B * self.dt[k]))
        else:
            sig = np.zeros(sc.ns)
        sig = np.ascontiguousarray(sig, np.float64)
        _lib.check(self.lib.mgx_batch_set_sigma(self.handle, k, _lib.dptr(sig)), "mgx_batch_set_sigma")

    def set_temperature(self, k, T):
        self.T[k] = float(T)
        self._push_sigma(k)

    def set_field(self, k, B):
        self.systems[k].set_field(B)
        self.models[k].sync_field()
        _lib.check(self.lib.mgx_batch_sync_models(self.handle), "mgx_batch_sync_models")

    # ------------------------------------------------------------------ spins
    def block(self, k):
        """(3, N_k) lattice-layout view of system k's spins on the device."""
        a, b = int(self.offsets[k]), int(self.offsets[k + 1])
        return self.e[3 * a:3 * b].view(3, b - a)

    def set_spins(self, spins):
        for k, e in enumerate(spins):
            self.models[k].to_lattice(e, out=self.block(k))

    def spins(self, k):
        """(N_k, 3) spins of system k in magex site order (device tensor)."""
        return self.models[k].from_lattice(self.block(k))

    # ------------------------------------------------------------------ stepping
    def step(self):
        noise_ptr = None
        if self.noise == "host":
            if self._noise is None:
                self._noise = torch.zeros_like(self.e)
            for k in range(self.nsys):
                g = self._rngs[k].normal(size=(self.systems[k].N, 3)) if self.T[k] > 0 else \
                    np.zeros((self.systems[k].N, 3))
                a, b = int(self.offsets[k]), int(self.offsets[k + 1])
                self.models[k].to_lattice(g, out=self._noise[3 * a:3 * b].view(3, b - a))
            noise_ptr = C.c_void_p(self._noise.data_ptr())
        _lib.check(self.lib.mgx_batch_step(self.handle, C.c_void_p(self.e.data_ptr()), noise_ptr,
                                           C.c_uint64(self._step_index), stream_ptr()), "mgx_batch_step")
        self._step_index += 1
        self.time += self.dt[0]

    def run(self, steps, graph_chunk=50):
        """steps steps of every system; graph_chunk > 0 replays a CUDA graph of that many steps."""
        steps = int(steps)
        if self.noise == "host":
            for _ in range(steps):
                self.step()
            return
        _lib.check(self.lib.mgx_batch_run(self.handle, C.c_void_p(self.e.data_ptr()), C.c_int64(steps),
                                          C.c_uint64(self._step_index), C.c_int32(int(graph_chunk or 0)),
                                          stream_ptr()), "mgx_batch_run")
        self._step_index += steps
        self.time += self.dt[0] * steps

    def set_launch(self, threads, ctas_per_sm):
        _lib.check(self.lib.mgx_batch_set_launch(self.handle, int(threads), int(ctas_per_sm)), "mgx_batch_set_launch")
        self.launch = (int(threads), int(ctas_per_sm))

    def autotune(self, steps=4, candidates=None, log=None):
        """Pick (threads per tile, resident CTAs per SM) by timing `steps` steps of each candidate on a
        copy of the spins (the state is restored afterwards).  Returns the chosen pair and the timings."""
        if candidates is None:
            candidates = [(t, c) for t in (128, 256, 512) for c in (0, 2, 4, 8)]
        saved = self.e.clone()
        saved_index = self._step_index
        timings = {}
        stream = torch.cuda.current_stream()
        for t, c in candidates:
            try:
                self.set_launch(t, c)
            except ValueError:
                continue
            _lib.check(self.lib.mgx_batch_run(self.handle, C.c_void_p(self.e.data_ptr()), 1, 0, 0, stream_ptr()),
                       "autotune warm-up")
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            _lib.check(self.lib.mgx_batch_run(self.handle, C.c_void_p(self.e.data_ptr()), steps, 0, 0, stream_ptr()),
                       "autotune")
            e1.record(stream)
            e1.synchronize()
            timings[(t, c)] = e0.elapsed_time(e1) / steps
            if log:
                log(f"  autotune threads={t:4d} ctas/SM={c}: {timings[(t, c)]:.4f} ms/step")
        best = min(timings, key=timings.get)
        self.set_launch(*best)
        self.e.copy_(saved)
        self._step_index = saved_index
        return best, timings

    # ------------------------------------------------------------------ observables
    def observables(self):
        """(nsys, 8) numpy: E (meV), sum e (3), sum s e (3), max torque (T) per system."""
        _lib.check(self.lib.mgx_batch_observables(self.handle, C.c_void_p(self.e.data_ptr()),
                                                  C.c_void_p(self._obs.data_ptr()), stream_ptr()),
                   "mgx_batch_observables")
        return self._obs.cpu().numpy().copy()

    def rows(self):
        """Per-system table rows [t, E/N, <ex>, <ey>, <ez>, order parameter, max torque] (magex/llg.py:257)."""
        obs = self.observables()
        N = (self.offsets[1:] - self.offsets[:-1]).astype(float)
        return np.column_stack([np.full(self.nsys, self.time), obs[:, 0] / N, obs[:, 1] / N, obs[:, 2] / N,
                                obs[:, 3] / N, np.linalg.norm(obs[:, 4:7], axis=1) / N, obs[:, 7]])

    def set_triangles(self, triangles):
        """triangles: per system (tri_sites (T_k, 3) in magex site order, orient (T_k,))."""
        tris, ors, off = [], [], [0]
        for k, (tri, orient) in enumerate(triangles):
            sc = self.systems[k]
            tri = np.asarray(tri, np.int64).reshape(-1, 3)
            cell, s = tri // sc.ns, tri % sc.ns
            tris.append((s * sc.ncell + cell).astype(np.int32))
            ors.append(np.asarray(orient, np.float64).reshape(-1))
            off.append(off[-1] + len(tri))
        tri = np.ascontiguousarray(np.concatenate(tris).reshape(-1), np.int32)
        ori = np.ascontiguousarray(np.concatenate(ors), np.float64)
        off = np.ascontiguousarray(off, np.int64)
        _lib.check(self.lib.mgx_batch_set_triangles(self.handle, _lib.iptr(tri), _lib.dptr(ori),
                                                    off.ctypes.data_as(C.POINTER(C.c_int64))),
                   "mgx_batch_set_triangles")

    def topological_charge(self):
        """(nsys,) numpy skyrmion numbers of the triangle lists set with set_triangles."""
        _lib.check(self.lib.mgx_batch_topological_charge(self.handle, C.c_void_p(self.e.data_ptr()),
                                                         C.c_void_p(self._Q.data_ptr()), stream_ptr()),
                   "mgx_batch_topological_charge")
        return self._Q.cpu().numpy().copy()
