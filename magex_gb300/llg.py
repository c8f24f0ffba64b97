"""GB300 drop-in for magex's stochastic LLG integrator (``magex.llg.LLGSolver``, heun / depondt).

    from magex_gb300 import LLGSolver            # or GB300LLG
    sol = LLGSolver(system, alpha=0.1, dt=1e-4, temperature=300, seed=1)
    e, table, snaps = sol.run(e0, steps=10000, output_every=100)

Same constructor, ``step``, ``run``, ``max_torque``, ``time`` / ``T`` / ``dt`` attributes and table
columns as magex ``magex/llg.py:48-283``.  The spins stay on the GPU for the whole ``run`` and every
Heun step is two fused sm_103a kernels (libmgx: ``mgx_llg_step`` / ``mgx_llg_run``); observables
rows are computed on the device by ``mgx_observables``.

Arithmetic (``precision=``): "fp64" runs everything in FP64.  "fp64_fixed" keeps every
floating-point operation FP64 and evaluates the exchange and on-site sums exactly on 56-bit
fixed-point spins and couplings (INT32 pipe): its only extra error, the 2^-57 quantisation of the
inputs, is below the rounding of an FP64 multiply-add chain, and it is 3.5x faster on GB300, whose
FP64 units run at 1/61 of its FP32 rate.  "auto" (default) is "fp64_fixed" for the models that form
supports (lattice stencils with per-sublattice moments and single-ion tensors, uniform damping and
temperature, no spin-orbit torque) where it is faster (at least 2^15 sites, couplings beyond
isotropic numbers) and "fp64" otherwise; a
solver on "auto" moves to an FP64 plan when field hooks (field_func, extra_field) are first used.
Two reduced forms keep the spins, the integration and the renormalisation in FP64 and move the rest
off the FP64 pipe (Heun: field and right-hand side on compensated FP32 pairs): "df32" evaluates the
exchange sum on compensated FP32 pairs (~44 significant bits), "int48" as exact integer products and
sums of 48-bit fixed-point couplings and spins.  Every form stays within the per-step parity
tolerance against magex (tests/test_gpu_df.py, tests/test_gpu_fixed_adversarial.py).

Thermal noise (``noise=``):
  "philox"  counter-based Philox4x32-10 keyed by (seed, site, step), generated inside the kernels
            (default; the trajectory differs from any magex backend, as magex's own numba and NumPy
            backends differ from each other, but the statistics are those of magex/llg.py:106-122);
  "host"    N(0,1) draws from ``numpy.random.default_rng(seed).normal(size=(N, 3))`` once per step,
            exactly the stream of magex's NumPy path (magex/llg.py:69,119): trajectories then
            reproduce magex's step for step.
"""
from __future__ import annotations

import ctypes as C
import time as _time

import numpy as np
import torch

from . import _lib
from .constants import GAMMA, K_B, MU_B
from .device import DeviceModel, stream_ptr, supercell_from_system

INTEGRATORS = ("heun", "rk4", "depondt", "sib", "euler")   # the names magex accepts (magex/llg.py:45)
_SUPPORTED = {"heun": _lib.HEUN, "depondt": _lib.DEPONDT}


def _philox_key(seed):
    ss = np.random.SeedSequence(None if seed is None else int(seed))
    return int(ss.generate_state(1, dtype=np.uint64)[0])



def llg_rhs(e, B, alpha, precession=True):
    """de/dt (1/ps) = -gamma / (1 + alpha^2) [e x B + alpha e x (e x B)] for (N, 3) spins and fields
    (host NumPy, magex/llg.py:21-28; the kernels evaluate the same expression per site)."""
    pre = -GAMMA / (1.0 + alpha * alpha)
    exB = np.cross(e, B)
    out = alpha * np.cross(e, exB)
    if precession:
        out = out + exB
    return pre * out


#: arithmetic forms of the step (precision=...), see the module docstring
PRECISIONS = {"fp64": _lib.PRECISION_FP64, "df32": _lib.PRECISION_DF32_GATHER, "int48": _lib.PRECISION_INT48_GATHER,
              "fp64_fixed": _lib.PRECISION_FP64_FIXED_GATHER}


#: below this many sites a step is bound by the latency of one thread's dependent chain, which the
#: longer integer gather lengthens: "auto" keeps the FP64 plan there (measured on GB300: the FP64 step
#: is faster up to ~16k sites for two-site bcc and triangular films)
AUTO_FIXED_MIN_SITES = 1 << 15


def fixed_point_eligible(sc, alpha=0.1, sot=None):
    """True when the exact fixed-point sum form (fp64_fixed) supports the system: a lattice stencil
    of fewer than 2^31 sites with per-sublattice moments and single-ion tensors, uniform damping and
    temperature, no extra energy terms (biquadratic, four-spin) and no spin-orbit torque.  Cubic and
    higher-uniaxial anisotropy are evaluated in FP64 beside the fixed-point sum."""
    from .lattice import Supercell
    if not isinstance(sc, Supercell) or sc.N >= 2 ** 31 or sot:
        return False
    if np.ndim(alpha) or getattr(sc, "alpha_site", None) is not None or getattr(sc, "site_T", None) is not None:
        return False
    if sc.A_site is not None or sc.mu_site is not None or getattr(sc, "terms", None):
        return False
    if len(sc.bond_src) and np.bincount(np.asarray(sc.bond_src)).max() > 127:
        return False                     # the 56-bit accumulators take at most 127 couplings per site
    return not sc.has_higher


def auto_fixed(sc, alpha=0.1, sot=None):
    """What precision="auto" picks: the fixed-point sum form where it is supported and faster, i.e.
    for lattices of at least AUTO_FIXED_MIN_SITES sites whose couplings are not plain isotropic
    numbers (an isotropic stencil costs the FP64 gather one multiply-add per component and neighbour,
    the fixed-point sum always nine products of a full tensor; measured: FP64 stays faster for the
    isotropic simple-cubic model up to 262k sites)."""
    return fixed_point_eligible(sc, alpha, sot) and sc.N >= AUTO_FIXED_MIN_SITES and int(sc.width) != 1

class GB300LLG:
    """Stochastic Heun / Depondt LLG on one GB300, with the API of magex ``LLGSolver``."""

    def __init__(self, system, alpha=0.1, dt=1e-3, temperature=0.0, seed=None, precession=True,
                 thermostat="classical", integrator="heun", stt=None, sot=None, backend="gb300",
                 noise="philox", precision="auto", device=None):
        if integrator not in INTEGRATORS:
            raise ValueError(f"integrator must be one of {INTEGRATORS}")
        if integrator not in _SUPPORTED:
            raise NotImplementedError(f"integrator '{integrator}' is not implemented by the GB300 kernels "
                                      "(heun and depondt are)")
        if thermostat != "classical":
            raise NotImplementedError("the quantum thermostat is not implemented by the GB300 kernels")
        if stt:
            raise NotImplementedError("spin-transfer torque (spin-current gradients) is not implemented by the GB300 kernels")
        if sot and precision not in ("fp64", "auto"):
            raise NotImplementedError("spin-orbit torque needs precision='fp64'")
        if backend not in ("gb300", "auto"):
            raise ValueError("backend must be 'gb300'")
        if noise not in ("philox", "host"):
            raise ValueError("noise must be 'philox' or 'host'")
        if precision not in PRECISIONS and precision != "auto":
            raise ValueError(f"precision must be 'auto' or one of {sorted(PRECISIONS)}")
        self.sys = system
        self.sc = supercell_from_system(system)
        self.auto_precision = precision == "auto"
        if self.auto_precision:
            precision = "fp64_fixed" if auto_fixed(self.sc, alpha, sot) else "fp64"
        self.precision = precision
        self.model = DeviceModel(self.sc, device)
        if system is not self.sc:
            self.model.field_owner = system          # follow SpinSystem.set_field (magex/llg.py:327)
        self.device = self.model.device
        N = self.sc.N
        a = getattr(self.sc, "alpha_site", None)
        self.alpha = np.asarray(a if (a is not None and np.isscalar(alpha)) else alpha, float)
        if self.alpha.ndim and a is not None and np.isscalar(alpha):
            self.alpha = np.where(np.isnan(self.alpha), float(alpha), self.alpha)
        self.dt = float(dt)
        self.T = float(temperature)
        self.seed = seed
        self.rng = np.random.default_rng(seed)
        self.precession = bool(precession)
        self.thermostat = thermostat
        self.integrator = integrator
        self.noise = noise
        self.time = 0.0
        self.field_func = None
        self.extra_field = None
        self._step_index = 0
        p = _lib.LLGParams()
        p.dt = self.dt
        if self.alpha.ndim:
            if self.alpha.shape != (N,):
                raise ValueError(f"alpha array must have shape ({N},)")
            al = np.ascontiguousarray(self.alpha, np.float64)
            p.alpha, p.alpha_site = 0.0, _lib.dptr(al)
        else:
            al = None
            p.alpha = float(self.alpha)
        p.precession = int(self.precession)
        p.integrator = _SUPPORTED[integrator]
        p.noise = _lib.NOISE_HOST if noise == "host" else _lib.NOISE_PHILOX
        p.seed = _philox_key(seed)
        p.precision = PRECISIONS[precision]
        self._params, self._alpha_keep = p, al
        self.handle = self._create_plan(p)
        self.sot = None
        if sot:
            # magex/llg.py:84-86: p normalised, damping-like and field-like amplitudes in tesla
            pv = np.asarray(sot.get("p", [0, 1, 0]), float)
            self.sot = (pv / np.linalg.norm(pv), float(sot.get("B_DL", 0.0)), float(sot.get("B_FL", 0.0)))
            _lib.check(self.model.lib.mgx_llg_set_sot(self.handle, _lib.dptr(np.ascontiguousarray(pv)), self.sot[1],
                                                      self.sot[2]), "mgx_llg_set_sot")
        self._sigma_key = None
        self._noisy = False
        self._noise_lat = None
        self._lat = None

    def _create_plan(self, p):
        h = C.c_void_p()
        with torch.cuda.device(self.device):
            _lib.check(self.model.lib.mgx_llg_create(self.model.handle, C.byref(p), C.byref(h)), "mgx_llg_create")
        return h

    def _ensure_fp64_plan(self):
        """A solver on precision "auto" with the fixed-point form moves to an FP64 plan (same seed,
        parameters and step counter) the first time field hooks are used: the per-site hook field
        is an input of the FP64 kernels only."""
        if self.precision == "fp64" or not self.auto_precision:
            return
        self._params.precision = PRECISIONS["fp64"]
        h = self._create_plan(self._params)
        old, self.handle = self.handle, h
        self.model.lib.mgx_llg_destroy(old)
        self.precision = "fp64"
        self._sigma_key = None

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            try:
                self.model.lib.mgx_llg_destroy(h)
            except Exception:
                pass
            self.handle = None

    # ------------------------------------------------------------------ thermal amplitude
    def _site_T(self):
        sT = getattr(self.sc, "site_T", None)
        if sT is None:
            return None
        return np.where(np.isnan(sT), self.T, sT)

    def _update_sigma(self):
        """sigma_i = sqrt(2 alpha_i k_B T_i / (gamma mu_i mu_B dt)) (magex/llg.py:111), pushed to the plan
        whenever T, dt or the site temperatures change."""
        sT = getattr(self.sc, "site_T", None)
        key = (self.T, id(sT), self.dt)
        if key == self._sigma_key:
            return
        self._sigma_key = key
        self._noisy = self.T > 0 or sT is not None
        lib, sc = self.model.lib, self.sc
        if not self._noisy:
            _lib.check(lib.mgx_llg_set_sigma(self.handle, _lib.dptr(np.zeros(sc.ns)), None), "mgx_llg_set_sigma")
            return
        per_site = self.alpha.ndim or sT is not None or sc.mu_site is not None
        if per_site:
            T = self._site_T() if sT is not None else self.T
            sig = np.sqrt(2.0 * self.alpha * K_B * T / (GAMMA * sc.mu * MU_B * self.dt))
            sig = np.ascontiguousarray(np.broadcast_to(sig, (sc.N,)), np.float64)
            _lib.check(lib.mgx_llg_set_sigma(self.handle, None, _lib.dptr(sig)), "mgx_llg_set_sigma")
        else:
            sig = np.sqrt(2.0 * self.alpha * K_B * self.T / (GAMMA * sc.mu_sub * MU_B * self.dt))
            sig = np.ascontiguousarray(sig, np.float64)
            _lib.check(lib.mgx_llg_set_sigma(self.handle, _lib.dptr(sig), None), "mgx_llg_set_sigma")

    # ------------------------------------------------------------------ stepping on device
    def _has_callables(self):
        return self.field_func is not None or self.extra_field is not None

    def _check_supported_callables(self):
        if self._has_callables():
            raise NotImplementedError("field_func / extra_field: step with step_lattice / run_lattice / step / run")

    def _step_callables(self, lat, noise_ptr, stream):
        """One step with magex's field hooks (magex/llg.py:124-137,216-227): the predictor sees
        field_func(t) and extra_field(e), the corrector field_func(t + dt) and extra_field(ep).  A
        uniform (3,) field_func goes into the model's external field; (N, 3) fields are summed on the
        host into the plan's per-site field (mgx_llg_set_extra_field).  The kernels are the plain
        predictor and corrector."""
        lib, N = self.model.lib, self.sc.N
        B0 = np.asarray(self.model._B, float).copy()
        ep = C.c_void_p()
        _lib.check(lib.mgx_llg_predicted(self.handle, C.byref(ep)), "mgx_llg_predicted")
        try:
            for stage, t in ((0, self.time), (1, self.time + self.dt)):
                uni, site = None, None
                if self.field_func is not None:
                    f = np.asarray(self.field_func(t), float)
                    if f.size == 3:
                        uni = f.reshape(3)
                    else:
                        site = f.reshape(N, 3).copy()
                if self.extra_field is not None:
                    src = lat.data_ptr() if stage == 0 else ep.value
                    aos = torch.empty((N, 3), dtype=torch.float64, device=self.device)
                    _lib.check(lib.mgx_unpack_spins(self.model.handle, C.c_void_p(src), C.c_void_p(aos.data_ptr()),
                                                    stream_ptr(stream)), "mgx_unpack_spins")
                    xf = np.asarray(self.extra_field(aos.cpu().numpy()), float).reshape(N, 3)
                    site = xf if site is None else site + xf
                self.model.push_field(B0 + uni if uni is not None else B0)
                if site is not None:
                    self._xf_lat = self.model.to_lattice(site, out=getattr(self, "_xf_lat", None), stream=stream)
                    ptr = C.c_void_p(self._xf_lat.data_ptr())
                else:
                    ptr = None
                _lib.check(lib.mgx_llg_set_extra_field(self.handle, ptr), "mgx_llg_set_extra_field")
                _lib.check(lib.mgx_llg_stage(self.handle, C.c_int32(stage), C.c_void_p(lat.data_ptr()), noise_ptr,
                                             C.c_uint64(self._step_index), stream_ptr(stream)), "mgx_llg_stage")
        finally:
            self.model.push_field(B0)
            _lib.check(lib.mgx_llg_set_extra_field(self.handle, None), "mgx_llg_set_extra_field")
        self._advance()

    def _prepare_step(self, stream):
        """Field and thermal amplitudes up to date; the device noise pointer of this step (host-noise
        mode: this step's N(0,1) draws from the NumPy stream, packed to the lattice layout)."""
        self.model.sync_field()
        self._update_sigma()
        if self.noise != "host":
            return None
        if self._noisy:
            g = self.rng.normal(size=(self.sc.N, 3))
            self._noise_lat = self.model.to_lattice(g, out=self._noise_lat, stream=stream)
        elif self._noise_lat is None:
            # T = 0: magex draws nothing (magex/llg.py:107-108); a zero field is added
            self._noise_lat = torch.zeros((3, self.sc.N), dtype=torch.float64, device=self.device)
        return C.c_void_p(self._noise_lat.data_ptr())

    def _advance(self, nsteps=1):
        self._step_index += int(nsteps)
        t, dt = self.time, self.dt
        for _ in range(int(nsteps)):         # one addition per step, as magex/llg.py:196,213,247 accumulate
            t += dt
        self.time = t

    def step_lattice(self, lat, stream=None):
        """One step on device spins in the lattice layout ((3, N) float64, in place)."""
        if self._has_callables():
            self._ensure_fp64_plan()
        noise_ptr = self._prepare_step(stream)
        if self._has_callables():
            self._step_callables(lat, noise_ptr, stream)
            return lat
        _lib.check(self.model.lib.mgx_llg_step(self.handle, C.c_void_p(lat.data_ptr()), noise_ptr,
                                               C.c_uint64(self._step_index), stream_ptr(stream)), "mgx_llg_step")
        self._advance()
        return lat

    def step_host(self, e, out):
        """One step from host (N, 3) float64 spins `e` (CPU tensor, magex site order) into `out` (may be
        `e`): one library call (``mgx_llg_step_host``) whose copies overlap the stages when both
        tensors are pinned.  Returns `out` once it holds the result."""
        N = self.sc.N
        for name, t in (("e", e), ("out", out)):
            if t.is_cuda or t.dtype != torch.float64 or tuple(t.shape) != (N, 3) or not t.is_contiguous():
                raise ValueError(f"{name} must be a contiguous ({N}, 3) float64 CPU tensor")
        if self._has_callables():            # the hooks run between the stages: no overlapped copies
            lat = self.model.to_lattice(e, out=self._lat)
            self._lat = lat
            self.step_lattice(lat)
            out.copy_(self.model.from_lattice(lat))
            return out
        stream = torch.cuda.current_stream(self.device)
        noise_ptr = self._prepare_step(stream)
        _lib.check(self.model.lib.mgx_llg_step_host(self.handle, C.c_void_p(e.data_ptr()), C.c_void_p(out.data_ptr()),
                                                    noise_ptr, C.c_uint64(self._step_index), stream_ptr(stream)),
                   "mgx_llg_step_host")
        stream.synchronize()
        self._advance()
        return out

    def run_lattice(self, lat, nsteps, stream=None):
        """nsteps steps on device lattice-layout spins; Philox noise only (one library call)."""
        if self.noise == "host" or self._has_callables():
            for _ in range(int(nsteps)):
                self.step_lattice(lat, stream)
            return lat
        self.model.sync_field()
        self._update_sigma()
        _lib.check(self.model.lib.mgx_llg_run(self.handle, C.c_void_p(lat.data_ptr()), C.c_int64(int(nsteps)),
                                              C.c_uint64(self._step_index), stream_ptr(stream)), "mgx_llg_run")
        self._advance(nsteps)
        return lat

    def stage_lattice(self, lat, stage, stream=None):
        """Predictor (stage 0) or corrector (stage 1) half of a step on device lattice spins
        (Philox or no noise); the step counter and the time advance after the corrector."""
        if self.noise == "host":
            raise ValueError("stage_lattice needs in-kernel (philox) noise")
        self._check_supported_callables()
        if stage == 0:
            self.model.sync_field()
            self._update_sigma()
        _lib.check(self.model.lib.mgx_llg_stage(self.handle, C.c_int32(stage), C.c_void_p(lat.data_ptr()), None,
                                                C.c_uint64(self._step_index), stream_ptr(stream)), "mgx_llg_stage")
        if stage == 1:
            self._advance()
        return lat

    # ------------------------------------------------------------------ magex API
    def step(self, e, out=None):
        """One integration step; returns new spins (magex/llg.py:216).

        A numpy array in gives a new numpy array out (the input is not modified); an (N, 3) CUDA
        tensor gives a CUDA tensor; an (N, 3) CPU tensor (pinned: the copies overlap the step) gives
        a CPU tensor, written into ``out`` when given.  Host arrays go through one library call
        (``step_host``)."""
        N = self.sc.N
        if self._has_callables() or (isinstance(e, torch.Tensor) and e.is_cuda):
            on_device = isinstance(e, torch.Tensor) and e.is_cuda
            lat = self.model.to_lattice(e, out=self._lat)
            self._lat = lat
            self.step_lattice(lat)
            dev = self.model.from_lattice(lat, out=getattr(self, "_aos", None))
            self._aos = dev
            if on_device or isinstance(e, torch.Tensor):
                return dev.clone().to(e.device) if out is None else out.copy_(dev)
            return dev.cpu().numpy()
        if isinstance(e, torch.Tensor):
            src = e if (e.dtype == torch.float64 and e.is_contiguous()) else e.to(torch.float64).contiguous()
            if src.shape != (N, 3):
                raise ValueError(f"spins have shape {tuple(src.shape)}, expected {(N, 3)}")
            if out is None:
                out = torch.empty((N, 3), dtype=torch.float64, pin_memory=e.is_pinned())
            return self.step_host(src, out)
        a = np.ascontiguousarray(e, dtype=np.float64)
        src = torch.from_numpy(a if a.flags.writeable else a.copy())
        if src.shape != (N, 3):
            raise ValueError(f"spins have shape {tuple(src.shape)}, expected {(N, 3)}")
        return self.step_host(src, torch.empty((N, 3), dtype=torch.float64)).numpy()

    # ------------------------------------------------------------------ magex's host-side pieces
    @property
    def _a(self):
        return self.alpha[:, None] if self.alpha.ndim else self.alpha

    def thermal_field(self):
        """One draw of the thermal field b (N, 3) in tesla from the solver's NumPy generator, 0.0 at
        T = 0 (magex/llg.py:106-122): sigma = sqrt(2 alpha k_B T_i / (gamma mu_i mu_B dt)), zero on
        pinned sites.  The steps themselves draw their noise inside the kernels or, with noise="host",
        from this same generator."""
        sT = self._site_T()
        if self.T <= 0 and sT is None:
            return 0.0
        T = self.T if sT is None else sT
        sigma2 = 2.0 * self.alpha * K_B * T / (GAMMA * self.sc.mu * MU_B * self.dt)
        b = np.sqrt(sigma2)[:, None] * self.rng.normal(size=(self.sc.N, 3))
        pinned = getattr(self.sc, "pinned", None)
        if pinned is not None:
            b[np.asarray(pinned, bool)] = 0.0
        return b

    def field(self, e, t):
        """B (N, 3) in tesla at spins e and time t (magex/llg.py:124-137): the effective field (on the
        device) plus the spin-orbit torque fields, field_func(t) and extra_field(e); zero on pinned
        sites when any of those is present."""
        e = np.asarray(e, float)
        B = self.effective_field(e)
        extras = self.sot is not None or self._has_callables()
        if self.sot is not None:
            p, bdl, bfl = self.sot
            B = B + bdl * np.cross(e, p[None, :]) + bfl * p[None, :]
        if self.field_func is not None:
            B = B + self.field_func(t)
        if self.extra_field is not None:
            B = B + self.extra_field(e)
        pinned = getattr(self.sc, "pinned", None)
        if pinned is not None and extras:
            B[np.asarray(pinned, bool)] = 0.0
        return B

    def rhs(self, e, b, t):
        """Tangent de/dt (1/ps) at spins e, thermal field b and time t (magex/llg.py:138-151)."""
        return llg_rhs(np.asarray(e, float), self.field(e, t) + b, self._a, self.precession)

    # ------------------------------------------------------------------ checkpoint / resume
    def checkpoint(self, e, path):
        """Write spins and the solver's clock to an .npz: magex's spin-file keys (spins, positions,
        mu, sublattice, cell, supercell; magex/llg.py:292-296, so the file also serves as an
        ``init_spins("file")`` input) plus the time, the step counter that keys the Philox noise, the
        seed, the temperature and the state of the host noise generator.  magex itself saves only the
        spins (its time and generator state are lost); ``resume`` continues the run exactly."""
        import json
        if isinstance(e, torch.Tensor):
            e = e.detach().cpu().numpy()
        e = np.ascontiguousarray(e, np.float64).reshape(self.sc.N, 3)
        sc = self.sc
        geo = {"mu": sc.mu, "sublattice": sc.sublattice, "supercell": np.array(sc.L)}
        if hasattr(sc, "uc"):                       # lattice supercells; neighbour lists have no geometry
            geo.update(positions=sc.positions, cell=sc.uc.cell)
        np.savez_compressed(path, spins=e, **geo, time=self.time, step=self._step_index,
                            seed=-1 if self.seed is None else int(self.seed), temperature=self.T, dt=self.dt,
                            noise=self.noise, rng_state=json.dumps(self.rng.bit_generator.state))
        return path

    def resume(self, path):
        """Spins of a checkpoint written by ``checkpoint``; restores the time, the step counter, the
        temperature and the host generator, so that the continued trajectory equals the
        uninterrupted one bit for bit.  The solver must have the checkpoint's seed, time step and
        noise mode (the Philox key is fixed when the solver is created)."""
        import json
        with np.load(path) as z:
            seed = int(z["seed"])
            mine = -1 if self.seed is None else int(self.seed)
            if seed != mine or str(z["noise"]) != self.noise or float(z["dt"]) != self.dt:
                raise ValueError(f"checkpoint {path} was written by a solver with seed {seed}, noise "
                                 f"'{z['noise']}', dt {float(z['dt'])}; this one has seed {mine}, noise "
                                 f"'{self.noise}', dt {self.dt}")
            if z["spins"].shape != (self.sc.N, 3):
                raise ValueError(f"checkpoint spins have shape {z['spins'].shape}, expected {(self.sc.N, 3)}")
            e = np.array(z["spins"], np.float64)
            self.time = float(z["time"])
            self._step_index = int(z["step"])
            self.T = float(z["temperature"])
            self.rng.bit_generator.state = json.loads(str(z["rng_state"]))
        return e

    def _row(self, lat):
        obs = self.model.observables(lat).cpu().numpy()
        N = self.sc.N
        return [self.time, obs[0] / N, obs[1] / N, obs[2] / N, obs[3] / N,
                float(np.linalg.norm(obs[4:7]) / N), float(obs[7])]

    def max_torque(self, e):
        """max_i |e_i x B_eff,i| (T) of the system's effective field, without field_func / extra_field
        (magex/llg.py:250-252)."""
        return float(self.model.observables(self.model.to_lattice(e))[7].item())

    def effective_field(self, e):
        """B_eff (N, 3) in tesla (magex/spinmodel.py:471-473), computed on the device."""
        lat = self.model.to_lattice(e)
        B = self.model.effective_field(lat)
        out = self.model.from_lattice(B)
        return out if (isinstance(e, torch.Tensor) and e.is_cuda) else out.cpu().numpy()

    def energy(self, e, per_spin=False):
        """Total energy (meV) (magex/spinmodel.py:475-484), computed on the device."""
        E = float(self.model.observables(self.model.to_lattice(e))[0].item())
        return E / self.sc.N if per_spin else E

    def run(self, e, steps, output_every=100, snapshots=0, callback=None, torque_tol=None, log=None):
        """Integrate ``steps`` steps; returns (spins, table, snapshots) as magex/llg.py:254-283.

        table columns: t (ps), E/N (meV), <ex>, <ey>, <ez>, order parameter, max torque (T).
        Between output rows the steps run back to back on the device (one library call per
        interval when no callback or snapshot needs the spins on the host).
        """
        on_device = isinstance(e, torch.Tensor) and e.is_cuda
        steps = int(steps)
        output_every = max(1, int(output_every))
        rows, snaps = [], []
        snap_every = max(1, steps // snapshots) if snapshots else 0
        lat = self.model.to_lattice(e)
        t0 = _time.time()

        def host_spins():
            return self.model.from_lattice(lat).cpu().numpy()

        n = 0
        while n <= steps:
            if n % output_every == 0 or n == steps:
                rows.append(self._row(lat))
                tq = rows[-1][6]
                if log and (n % (output_every * 10) == 0 or n == steps):
                    m = rows[-1][2:5]
                    log(f"  step {n:8d}  t = {self.time:9.3f} ps  E/N = {rows[-1][1]: .6f} meV  "
                        f"m = ({m[0]: .3f},{m[1]: .3f},{m[2]: .3f})  |torque|max = {tq:.2e} T")
                if torque_tol is not None and self.T == 0 and tq < torque_tol and n > 0:
                    if log:
                        log(f"  converged: max torque {tq:.2e} T < {torque_tol:g} T after {n} steps")
                    break
            if snap_every and n % snap_every == 0:
                snaps.append((self.time, host_spins()))
            if callback:
                callback(n, host_spins())
            if n >= steps:
                break
            # advance to the next step at which the host needs something
            nxt = min(steps, (n // output_every + 1) * output_every)
            if snap_every:
                nxt = min(nxt, (n // snap_every + 1) * snap_every)
            if callback:
                nxt = n + 1
            self.run_lattice(lat, nxt - n)
            n = nxt
        if log:
            torch.cuda.synchronize(self.device)
            log(f"  LLG wall time {_time.time() - t0:.1f} s")
        out = self.model.from_lattice(lat)
        return (out if on_device else out.cpu().numpy()), np.array(rows), snaps


LLGSolver = GB300LLG
