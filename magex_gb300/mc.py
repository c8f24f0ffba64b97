"""Monte Carlo colour sweeps on the GB300: a drop-in for magex's ``MetropolisMC`` and its runs.

    from magex_gb300.mc import MetropolisMC          # same signature as magex.montecarlo.MetropolisMC
    mc = MetropolisMC(system, temperature=20.0, seed=1, sigma=0.6, overrelax=1, move="gaussian")
    e = mc.sweep(e)                                   # one sweep, in place, as magex
    a = mc.acceptance()

Sites are split into colour classes by magex's first-fit greedy colouring in site order
(``magex/montecarlo.py:35-48``, computed natively by ``mgx_colour_stencil`` / ``mgx_colour_graph``);
the classes, with pinned sites left out, are the update groups of ``magex/montecarlo.py:88-99``.  Each
class is one kernel launch (``mgx_mc_sweep``): trial move (Gaussian cone, uniform, heat bath, Hinzke
mixture), the energy change of ``magex/montecarlo.py:136-147`` and the Metropolis test, then the
over-relaxation passes about the exchange field.

``rng="philox"`` (default) draws inside the kernels from a counter-based stream keyed by
(seed, site, sweep, pass).  ``rng="host"`` draws on the host with ``numpy.random.default_rng(seed)``
in exactly the order of magex's NumPy sweep, so that a sweep reproduces magex's own trajectory.
"""
from __future__ import annotations

import ctypes as C
import time

import numpy as np
import torch

from . import _lib
from .constants import K_B
from .device import DeviceModel, stencil_desc, stream_ptr, supercell_from_system
from .lattice import NeighbourList

MOVES = {"gaussian": _lib.MC_GAUSSIAN, "uniform": _lib.MC_UNIFORM, "heatbath": _lib.MC_HEATBATH,
         "hinzke": _lib.MC_HINZKE}


def colouring(sc):
    """(colour (N,) int32, ncolours): magex's greedy colouring of the coupling graph of a Supercell
    or NeighbourList (host only; identical to magex.montecarlo.greedy_coloring on system.bonds)."""
    lib = _lib.load()
    col = np.empty(sc.N, np.int32)
    nc = C.c_int32()
    if isinstance(sc, NeighbourList):
        ptr = np.asarray(sc.ptr, np.int64)
        rows = np.repeat(np.arange(sc.N, dtype=np.int64), np.diff(ptr))
        cols = np.asarray(sc.nbr, np.int64)
        a = np.concatenate([rows, cols])
        b = np.concatenate([cols, rows])
        keep = a != b
        key = np.unique(a[keep] * sc.N + b[keep])
        src, dst = key // sc.N, (key % sc.N).astype(np.int32)
        sptr = np.zeros(sc.N + 1, np.int64)
        np.add.at(sptr, src + 1, 1)
        sptr = np.cumsum(sptr)
        dst = np.ascontiguousarray(dst)
        _lib.check(lib.mgx_colour_graph(sc.N, sptr.ctypes.data_as(C.POINTER(C.c_int64)), _lib.iptr(dst),
                                        _lib.iptr(col), C.byref(nc)), "mgx_colour_graph")
    else:
        d, keep = stencil_desc(sc)
        _lib.check(lib.mgx_colour_stencil(C.byref(d), _lib.iptr(col), C.byref(nc)), "mgx_colour_stencil")
        del keep
    return col, int(nc.value)


class MetropolisMC:
    """Metropolis / heat-bath colour sweeps on the GB300 (``magex/montecarlo.py:71-230``).

    Same arguments as magex; ``backend`` and ``dipolar_exact`` are accepted for signature
    compatibility (dipolar and other long-range terms raise NotImplementedError).  ``rng`` selects
    in-kernel Philox draws or magex's own NumPy stream; ``precision="fp64_fixed"`` evaluates the
    exchange field of the trial moves as an exact 56-bit fixed-point sum on the integer pipes (stencil
    models with per-sublattice A and mu; every floating-point operation stays FP64).  ``T`` and ``sigma`` may be reassigned between
    sweeps (annealing, magex/montecarlo.py:257-261)."""

    def __init__(self, system, temperature, seed=None, sigma=0.6, overrelax=1, move="gaussian",
                 backend="gb300", dipolar_exact="auto", rng="philox", precision="fp64", device=None):
        if move not in MOVES:
            raise ValueError(f"unknown move '{move}' (gaussian, uniform, heatbath, hinzke)")
        if rng not in ("philox", "host"):
            raise ValueError("rng must be 'philox' or 'host'")
        if precision not in ("fp64", "fp64_fixed"):
            raise ValueError("precision must be 'fp64' or 'fp64_fixed' (exchange field as an exact 56-bit "
                             "fixed-point sum, every floating-point operation FP64)")
        self.sys = system
        self.sc = supercell_from_system(system)
        self.move = move
        self.overrelax = int(overrelax)
        self.rng_mode = rng
        self.rng = np.random.default_rng(seed)
        self.model = DeviceModel(self.sc, device)
        self.model.field_owner = system if system is not self.sc else None
        self.device = self.model.device
        sc = self.sc
        col, nc = colouring(sc)
        pinned = None if getattr(sc, "pinned", None) is None else np.asarray(sc.pinned, bool)
        self.groups = []
        for c in range(nc):
            idx = np.flatnonzero(col == c)
            if pinned is not None:
                idx = idx[~pinned[idx]]
            if len(idx):
                self.groups.append(idx)
        self.ncolors = len(self.groups)
        sites = np.ascontiguousarray(np.concatenate(self.groups) if self.groups else np.zeros(0), np.int64)
        sizes = np.ascontiguousarray([len(g) for g in self.groups], np.int64)
        p = _lib.MCParams()
        p.move = MOVES[move]
        p.overrelax = self.overrelax
        p.rng = _lib.MC_RNG_HOST if rng == "host" else _lib.MC_RNG_PHILOX
        p.sigma = float(sigma)
        p.seed = int(np.random.SeedSequence(seed).generate_state(1, np.uint64)[0])
        p.precision = _lib.PRECISION_FP64_FIXED_GATHER if precision == "fp64_fixed" else _lib.PRECISION_FP64
        h = C.c_void_p()
        lib = _lib.load()
        with torch.cuda.device(self.device):
            _lib.check(lib.mgx_mc_create(self.model.handle, C.byref(p),
                                         sites.ctypes.data_as(C.POINTER(C.c_int64)),
                                         sizes.ctypes.data_as(C.POINTER(C.c_int64)), len(self.groups), C.byref(h)),
                       "mgx_mc_create")
        self.lib = lib
        self.handle = h
        self._sigma = float(sigma)
        self._T = float(temperature)
        self._beta_key = None
        self._hb = [True] * len(self.groups)
        self._sync_beta()

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            try:
                self.lib.mgx_mc_destroy(h)
            except Exception:
                pass
            self.handle = None

    # ------------------------------------------------------------------ parameters
    @property
    def T(self):
        return self._T

    @T.setter
    def T(self, value):
        self._T = float(value)

    @property
    def sigma(self):
        return self._sigma

    @sigma.setter
    def sigma(self, value):
        self._sigma = float(value)
        _lib.check(self.lib.mgx_mc_set_sigma(self.handle, self._sigma), "mgx_mc_set_sigma")

    def _beta_site(self):
        """Per-site beta (magex order) with site temperatures, else None (magex/montecarlo.py:149-154)."""
        sT = getattr(self.sys, "site_T", None)
        if sT is None:
            sT = getattr(self.sc, "site_T", None)
        if sT is None:
            return None
        T = np.where(np.isnan(sT), self._T, sT)
        return 1.0 / (K_B * np.maximum(T, 1e-9))

    def _sync_beta(self):
        bs = self._beta_site()
        key = (self._T, None if bs is None else bs.tobytes())
        if key == self._beta_key:
            return
        if bs is None:
            b = 1.0 / (K_B * self._T) if self._T > 0 else np.inf
            sub = np.full(self.sc.ns if not isinstance(self.sc, NeighbourList) else 1, b)
            _lib.check(self.lib.mgx_mc_set_beta(self.handle, _lib.dptr(sub), None), "mgx_mc_set_beta")
            self._hb = [bool(np.isfinite(b))] * len(self.groups)
        else:
            bs = np.ascontiguousarray(bs, np.float64)
            _lib.check(self.lib.mgx_mc_set_beta(self.handle, None, _lib.dptr(bs)), "mgx_mc_set_beta")
            self._hb = [bool(np.all(np.isfinite(bs[g]))) for g in self.groups]
        self._beta_key = key

    # ------------------------------------------------------------------ host draws (magex's NumPy order)
    def _host_draws(self):
        rng = self.rng
        out = []
        for g, idx in enumerate(self.groups):
            n = len(idx)
            if self.move == "heatbath" and self._hb[g]:
                out += [rng.random(n), rng.random(n)]             # magex/montecarlo.py:51-68 (u, phi)
            elif self.move == "hinzke":
                out += [rng.integers(0, 3, n).astype(np.float64), rng.normal(size=(n, 3)).ravel(),
                        rng.normal(size=(n, 3)).ravel()]          # magex/montecarlo.py:217-224
            else:
                out.append(rng.normal(size=(n, 3)).ravel())       # magex/montecarlo.py:225-226
            out.append(rng.random(n))                             # acceptance (magex/montecarlo.py:196)
        for _ in range(self.overrelax):
            for idx in self.groups:
                out.append(rng.random(len(idx)))                  # magex/montecarlo.py:208
        return np.concatenate(out) if out else np.zeros(0)

    # ------------------------------------------------------------------ sweeps
    def sweep_lattice(self, lat, nsweeps=1, stream=None):
        """nsweeps sweeps of device spins in the lattice layout ((3, N) float64 CUDA tensor)."""
        if lat.shape != (3, self.sc.N) or lat.dtype != torch.float64 or not lat.is_cuda:
            raise ValueError("lattice spins must be a (3, N) float64 CUDA tensor")
        self.model.sync_field()
        self._sync_beta()
        if self.rng_mode == "host":
            need = C.c_int64()
            _lib.check(self.lib.mgx_mc_host_draws(self.handle, C.byref(need)), "mgx_mc_host_draws")
            for _ in range(int(nsweeps)):
                draws = torch.as_tensor(self._host_draws(), device=lat.device)
                if draws.numel() != need.value:
                    raise RuntimeError(f"host draws: {draws.numel()} doubles prepared, the sweep reads {need.value}")
                _lib.check(self.lib.mgx_mc_sweep(self.handle, C.c_void_p(lat.data_ptr()), 1,
                                                 C.c_void_p(draws.data_ptr()), stream_ptr(stream)), "mgx_mc_sweep")
                torch.cuda.current_stream().synchronize() if stream is None else stream.synchronize()
            return lat
        _lib.check(self.lib.mgx_mc_sweep(self.handle, C.c_void_p(lat.data_ptr()), int(nsweeps), None,
                                         stream_ptr(stream)), "mgx_mc_sweep")
        return lat

    def sweep(self, e):
        """One sweep of e ((N, 3) numpy array or CUDA tensor, magex order), updated in place and
        returned, as magex/montecarlo.py:181-210."""
        if isinstance(e, torch.Tensor):
            lat = self.model.to_lattice(e)
            self.sweep_lattice(lat)
            e.copy_(self.model.from_lattice(lat).to(e.device))
            return e
        arr = np.asarray(e)
        if arr.shape != (self.sc.N, 3):
            raise ValueError(f"spins must have shape {(self.sc.N, 3)}, got {arr.shape}")
        lat = self.model.to_lattice(np.ascontiguousarray(arr, np.float64))
        self.sweep_lattice(lat)
        out = self.model.from_lattice(lat).cpu().numpy()
        if isinstance(e, np.ndarray) and e.dtype == np.float64 and e.flags.writeable:
            e[...] = out
            return e
        return out

    def counts(self, reset=False):
        """(accepted, tried) trial moves since the last reset (synchronises the stream)."""
        a, t = C.c_uint64(), C.c_uint64()
        _lib.check(self.lib.mgx_mc_counts(self.handle, C.byref(a), C.byref(t), int(bool(reset)), stream_ptr()),
                   "mgx_mc_counts")
        return int(a.value), int(t.value)

    @property
    def accepted(self):
        return self.counts()[0]

    @property
    def tried(self):
        return self.counts()[1]

    def acceptance(self, reset=True):
        """Accepted fraction of the trial moves since the last reset (magex/montecarlo.py:229-234)."""
        a, t = self.counts(reset)
        return a / max(t, 1)


GB300MC = MetropolisMC


# ---------------------------------------------------------------------- one (L, T) point and T_c
def _blocks_obs(E, m, N, kT):
    C_ = (np.mean(E ** 2) - np.mean(E) ** 2) / (N * kT ** 2)
    chi = N * (np.mean(m ** 2) - np.mean(m) ** 2) / kT
    U4 = 1 - np.mean(m ** 4) / (3 * np.mean(m ** 2) ** 2)
    return np.mean(E) / N, C_, np.mean(m), chi, U4


def point(args, rng="philox"):
    """One (system size, temperature) run with the arguments of magex/montecarlo.py:251-307 (_point):
    args = (uc, L, pbc, B, T, c, seed) with c holding sigma, overrelax, move, init, init_axis,
    therm_sweeps, meas_sweeps, sample_every (and keep_spins).  Thermalisation adapts sigma every 50
    sweeps towards 50 % acceptance; measurement samples E and the order vector on the device.  Returns
    the same row dictionary (E, C, m, chi, U4 per spin with 10-block errors, acceptance, sigma, ...)."""
    from .lattice import Supercell
    uc, L, pbc, B, T, c, seed = args
    if c.get("structure"):
        raise NotImplementedError("structure edits: build the system with magex.structure and pass it to "
                                  "MetropolisMC directly")
    system = Supercell(uc, L, pbc, B)
    mc = MetropolisMC(system, T, seed, c["sigma"], c["overrelax"], c.get("move", "gaussian"), rng=rng)
    e = system.init_spins(c["init"], c["init_axis"], seed)
    lat = mc.model.to_lattice(e)
    t0 = time.time()
    for n in range(c["therm_sweeps"]):
        mc.sweep_lattice(lat)
        if (n + 1) % 50 == 0:
            a = mc.acceptance()
            mc.sigma = float(np.clip(mc.sigma * 0.5 / max(1 - a, 0.05), 0.02, 4.0))
    mc.acceptance()
    N = system.N
    Es, ms, mvec = [], [], []
    for n in range(c["meas_sweeps"]):
        mc.sweep_lattice(lat)
        if n % c["sample_every"] == 0:
            o = mc.model.observables(lat).cpu().numpy()
            v = o[4:7] / N
            Es.append(o[0])
            mvec.append(v)
            ms.append(np.linalg.norm(v))
    acc = mc.acceptance()
    spins = mc.model.from_lattice(lat).cpu().numpy() if c.get("keep_spins") else None
    return _row_of(L, N, T, Es, ms, mvec, acc, mc.sigma, mc.ncolors, time.time() - t0, spins)


def _row_of(L, N, T, Es, ms, mvec, acc, sigma, ncolors, seconds, spins):
    """Row dictionary of one (L, T) point from its samples (magex/montecarlo.py:274-291)."""
    E, m = np.array(Es), np.array(ms)
    kT = K_B * T
    full = _blocks_obs(E, m, N, kT)
    nb = 10
    n = len(E) // nb
    if n > 2:
        bl = np.array([_blocks_obs(E[k * n:(k + 1) * n], m[k * n:(k + 1) * n], N, kT) for k in range(nb)])
        err = bl.std(0, ddof=1) / np.sqrt(nb)
    else:
        err = np.zeros(5)
    return dict(L=list(L), N=N, T=T, E=full[0], C=full[1], m=full[2], chi=full[3], U4=full[4],
                dE=err[0], dC=err[1], dm=err[2], dchi=err[3], dU4=err[4], acceptance=acc,
                sigma=sigma, ncolors=ncolors, mvec=np.mean(mvec, 0).tolist(), seconds=seconds, spins=spins)


def _ensemble_key(job):
    uc, L, pbc, B, T, c, seed = job
    return (id(uc), tuple(int(x) for x in L), tuple(bool(x) for x in pbc),
            tuple(float(x) for x in np.asarray(B, float).ravel()), id(c))


def points(jobs, max_chains=4096):
    """Many (L, T) points at once: the rows of ``[point(job) for job in jobs]``, bit for bit.

    magex runs its points as separate processes (magex/montecarlo.py:390-401).  On one GPU the points
    that share a lattice (the same uc, L, pbc, B and run configuration c; temperatures and seeds
    differ) run as one ensemble (``mgx_mc_set_chains``): every pass of a sweep is one launch over the
    class's sites of all chains, the cone widths adapt on the device every 50 thermalisation sweeps,
    and the samples of E and the order vector are reduced into a device buffer, read once at the end.
    The ensembles of different lattices (e.g. the sizes of a T_c scan) run concurrently, each on its
    own CUDA stream.  Each chain's trajectory is that of its own ``point``.  Points with T = 0 or
    structure edits run one by one.  ``seconds`` of an ensemble's rows is its wall time divided by its
    number of chains."""
    from .lattice import Supercell
    jobs = list(jobs)
    rows = [None] * len(jobs)
    groups = {}
    for i, job in enumerate(jobs):
        c, T = job[5], float(job[4])
        if c.get("structure") or not T > 0:
            rows[i] = point(job)
            continue
        groups.setdefault(_ensemble_key(job), []).append(i)
    parts = [idxs[k:k + max_chains] for idxs in groups.values() for k in range(0, len(idxs), max_chains)]
    runs = [(part, _ensemble([jobs[i] for i in part], Supercell), torch.cuda.Stream()) for part in parts]
    # round-robin: each generator enqueues a batch of sweeps on its stream and yields
    while runs:
        left = []
        for part, gen, stream in runs:
            with torch.cuda.stream(stream):
                try:
                    next(gen)
                    left.append((part, gen, stream))
                except StopIteration as done:
                    for i, row in zip(part, done.value):
                        rows[i] = row
        runs = left
    return rows


def _ensemble(jobs, Supercell):
    """Generator running one ensemble on the current stream; yields after each batch of enqueued
    work and returns the rows."""
    uc, L, pbc, B, _, c, _ = jobs[0]
    n = len(jobs)
    Ts = [float(j[4]) for j in jobs]
    seeds = [j[6] for j in jobs]
    system = Supercell(uc, L, pbc, B)
    N = system.N
    mc = MetropolisMC(system, Ts[0], seeds[0], c["sigma"], c["overrelax"], c.get("move", "gaussian"))
    lib, h = mc.lib, mc.handle
    keys = np.array([np.random.SeedSequence(s).generate_state(1, np.uint64)[0] for s in seeds], np.uint64)
    beta = np.array([1.0 / (K_B * T) for T in Ts], np.float64)
    sig0 = np.full(n, float(c["sigma"]), np.float64)
    _lib.check(lib.mgx_mc_set_chains(h, n, keys.ctypes.data_as(C.c_void_p), _lib.dptr(beta), _lib.dptr(sig0)),
               "mgx_mc_set_chains")
    lat = torch.stack([mc.model.to_lattice(system.init_spins(c["init"], c["init_axis"], s)) for s in seeds])
    mc.model.sync_field()
    ptr = C.c_void_p(lat.data_ptr())

    def sweep(k):
        if k > 0:
            _lib.check(lib.mgx_mc_sweep(h, ptr, int(k), None, stream_ptr()), "mgx_mc_sweep")

    def counts(reset):
        acc = np.zeros(n, np.uint64)
        tried = C.c_uint64()
        sig = np.zeros(n, np.float64)
        _lib.check(lib.mgx_mc_chain_counts(h, acc.ctypes.data_as(C.c_void_p), C.byref(tried), _lib.dptr(sig),
                                           int(reset), stream_ptr()), "mgx_mc_chain_counts")
        return acc, int(tried.value), sig

    t0 = time.time()
    yield
    therm = int(c["therm_sweeps"])
    for _ in range(therm // 50):                 # sigma adapts after sweeps 50, 100, ... (as point())
        sweep(50)
        _lib.check(lib.mgx_mc_adapt_sigma(h, stream_ptr()), "mgx_mc_adapt_sigma")
        yield
    sweep(therm % 50)
    counts(True)
    meas, every = int(c["meas_sweeps"]), int(c["sample_every"])
    nsamp = (meas + every - 1) // every if meas > 0 else 0
    obs = torch.empty((max(nsamp, 1), n, 8), dtype=torch.float64, device=lat.device)
    done = 0
    for j in range(nsamp):                       # samples after sweeps 1, 1 + every, 1 + 2 every, ...
        sweep(j * every + 1 - done)
        done = j * every + 1
        _lib.check(lib.mgx_observables_n(mc.model.handle, ptr, n, C.c_void_p(obs[j].data_ptr()), stream_ptr()),
                   "mgx_observables_n")
        if j % 10 == 9:
            yield
    sweep(meas - done)
    acc, tried, sig = counts(True)
    o = obs[:nsamp].cpu().numpy()
    seconds = (time.time() - t0) / n
    rows = []
    for k in range(n):
        v = o[:, k, 4:7] / N
        spins = mc.model.from_lattice(lat[k]).cpu().numpy() if c.get("keep_spins") else None
        rows.append(_row_of(L, N, jobs[k][4], list(o[:, k, 0]), [np.linalg.norm(x) for x in v], list(v),
                            int(acc[k]) / max(tried, 1), float(sig[k]), mc.ncolors, seconds, spins))
    return rows


def parallel_tempering(system, temperatures, therm_sweeps=2000, meas_sweeps=4000, sample_every=2, swap_every=5,
                       seed=1, init="reference", init_axis=(0, 0, 1), sigma=0.6, overrelax=1, log=None):
    """Replica exchange with the arguments and return value of magex/advanced_mc.py:38-95: replicas at
    temperatures T_1 < ... < T_M sweep, every ``swap_every`` sweeps neighbouring pairs (even pairs,
    then odd, alternating) exchange configurations with probability min(1, exp[(b_k - b_k+1)
    (E_k - E_k+1)]) drawn from ``default_rng(seed)`` as magex does; returns (rows like point(),
    swap acceptance per neighbouring pair).

    The replicas are the chains of one ensemble (``mgx_mc_set_chains``, Philox key of seed + 17 k as
    magex seeds replica k): every pass of a sweep is one launch for all of them, cone widths adapt on
    the device, a swap exchanges the two chains' spin blocks on the device, and the replica energies
    for the swap decisions come back in one ``mgx_observables_n`` read."""
    Ts = np.array(sorted(float(t) for t in temperatures))
    M = len(Ts)
    if M < 1 or not np.all(Ts > 0):
        raise ValueError("parallel tempering needs temperatures > 0")
    rng = np.random.default_rng(seed)
    mc = MetropolisMC(system, Ts[0], seed, sigma, overrelax)
    sc, lib, h = mc.sc, mc.lib, mc.handle
    N = sc.N
    keys = np.array([np.random.SeedSequence(seed + 17 * k).generate_state(1, np.uint64)[0] for k in range(M)],
                    np.uint64)
    beta = np.array([1.0 / (K_B * T) for T in Ts], np.float64)
    _lib.check(lib.mgx_mc_set_chains(h, M, keys.ctypes.data_as(C.c_void_p), _lib.dptr(beta),
                                     _lib.dptr(np.full(M, float(sigma)))), "mgx_mc_set_chains")
    lat = torch.stack([mc.model.to_lattice(sc.init_spins(init, init_axis, seed + k)) for k in range(M)])
    mc.model.sync_field()
    st = stream_ptr()
    ptr = C.c_void_p(lat.data_ptr())
    total = int(therm_sweeps) + int(meas_sweeps)
    nsamp = len(range(0, int(meas_sweeps), int(sample_every)))
    samples = torch.empty((max(nsamp, 1), M, 8), dtype=torch.float64, device=lat.device)
    energies = torch.empty((M, 8), dtype=torch.float64, device=lat.device)
    swaps_try, swaps_acc = np.zeros(max(M - 1, 0)), np.zeros(max(M - 1, 0))
    t0 = time.time()
    j = 0
    for n in range(total):
        _lib.check(lib.mgx_mc_sweep(h, ptr, 1, None, st), "mgx_mc_sweep")
        if n < therm_sweeps and (n + 1) % 50 == 0:
            _lib.check(lib.mgx_mc_adapt_sigma(h, st), "mgx_mc_adapt_sigma")
        if (n + 1) % swap_every == 0 and M > 1:
            _lib.check(lib.mgx_observables_n(mc.model.handle, ptr, M, C.c_void_p(energies.data_ptr()), st),
                       "mgx_observables_n")
            E = energies[:, 0].cpu().numpy().copy()
            perm = list(range(M))
            for k in range((n // swap_every) % 2, M - 1, 2):
                d = (1 / (K_B * Ts[k]) - 1 / (K_B * Ts[k + 1])) * (E[k] - E[k + 1])
                swaps_try[k] += 1
                if d >= 0 or rng.random() < np.exp(d):
                    perm[k], perm[k + 1] = perm[k + 1], perm[k]
                    E[k], E[k + 1] = E[k + 1], E[k]
                    swaps_acc[k] += 1
            if perm != list(range(M)):
                lat.copy_(lat[perm])                 # configurations change places, temperatures stay
        if n >= therm_sweeps and (n - therm_sweeps) % sample_every == 0:
            _lib.check(lib.mgx_observables_n(mc.model.handle, ptr, M, C.c_void_p(samples[j].data_ptr()), st),
                       "mgx_observables_n")
            j += 1
    acc = np.zeros(M, np.uint64)
    tried = C.c_uint64()
    sig = np.zeros(M, np.float64)
    _lib.check(lib.mgx_mc_chain_counts(h, acc.ctypes.data_as(C.c_void_p), C.byref(tried), _lib.dptr(sig), 0, st),
               "mgx_mc_chain_counts")
    o = samples[:nsamp].cpu().numpy()
    L = list(getattr(system, "L", sc.L))
    rows = []
    for k, T in enumerate(Ts):
        v = o[:, k, 4:7] / N
        row = _row_of(L, N, float(T), list(o[:, k, 0]), [np.linalg.norm(x) for x in v], list(v),
                      int(acc[k]) / max(int(tried.value), 1), float(sig[k]), mc.ncolors, time.time() - t0, None)
        row["mvec"] = [0, 0, 0]                     # as magex/advanced_mc.py:88
        row.pop("spins")
        rows.append(row)
    swap = (swaps_acc / np.maximum(swaps_try, 1)).tolist()
    if log:
        log(f"  parallel tempering L={L}: {M} replicas, swap acceptance {np.round(swap, 2).tolist()}, "
            f"{time.time() - t0:.1f} s")
    return rows, swap


def _peak(T, y):
    """Peak of y(T): vertex of the parabola through the maximum and its neighbours when it lies
    between them, else the sampled maximum."""
    k = int(np.argmax(y))
    if 0 < k < len(T) - 1:
        a, b, _ = np.polyfit(T[k - 1:k + 2], y[k - 1:k + 2], 2)
        if a < 0:
            t = -b / (2 * a)
            if T[k - 1] <= t <= T[k + 1]:
                return float(t)
    return float(T[k])


def _crossings(T, u_small, u_large):
    """Temperatures where the larger system's Binder cumulant falls below the smaller one's
    (sign change of u_small - u_large from - to +), by linear interpolation."""
    d = np.asarray(u_small) - np.asarray(u_large)
    out = []
    for k in range(len(T) - 1):
        if d[k] < 0 <= d[k + 1]:
            out.append(T[k] - d[k] * (T[k + 1] - T[k]) / (d[k + 1] - d[k]))
    return [float(x) for x in out]


def estimate_tc(rows):
    """Ordering temperature from point() rows of several sizes (magex/montecarlo.py:310-347):
    chi and C peaks per size, Binder crossings of successive sizes (kept where U4 of the smaller size
    lies in (0.47, 0.67)), T_c = the crossing of the two largest sizes nearest the chi peak of the
    largest size, else that chi peak."""
    sizes = sorted({tuple(r["L"]) for r in rows}, key=lambda L: np.prod(L))
    est = dict(chi_peak={}, C_peak={}, binder=[])
    by = {L: sorted([r for r in rows if tuple(r["L"]) == L], key=lambda r: r["T"]) for L in sizes}
    for L in sizes:
        T = np.array([r["T"] for r in by[L]])
        est["chi_peak"][str(L)] = _peak(T, np.array([r["chi"] for r in by[L]]))
        est["C_peak"][str(L)] = _peak(T, np.array([r["C"] for r in by[L]]))
    for L1, L2 in zip(sizes[:-1], sizes[1:]):
        T1, T2 = [r["T"] for r in by[L1]], [r["T"] for r in by[L2]]
        if T1 != T2:
            continue
        u1, u2 = [r["U4"] for r in by[L1]], [r["U4"] for r in by[L2]]
        good = [x for x in _crossings(np.array(T1), u1, u2) if 0.47 < np.interp(x, T1, u1) < 0.67]
        est["binder"].append(dict(sizes=[list(L1), list(L2)], T=good))
    big = str(sizes[-1])
    Tchi = est["chi_peak"][big]
    if est["binder"] and est["binder"][-1]["T"]:
        est["Tc"] = float(min(est["binder"][-1]["T"], key=lambda x: abs(x - Tchi)))
        est["method"] = "Binder-cumulant crossing of the two largest sizes"
    else:
        est["Tc"] = Tchi
        est["method"] = f"susceptibility peak of the largest size {sizes[-1]}"
    return est
