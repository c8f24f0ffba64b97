"""Differentiable LLG trajectories: the hand-written adjoint of the Heun step behind torch.autograd.

    adj = AdjointLLG(sc, groups, alpha=0.3, dt=1e-4, seg_steps=100)
    eT = llg_trajectory(adj, e0, T, A, B, nsteps=2000)       # torch tensors, autograd-aware
    loss = ((eT - target) ** 2).sum()
    loss.backward()                                           # e0.grad, T.grad, A.grad, B.grad

The couplings of the supercell stencil are parameterised by a few 3x3 tensors ``T[g]``: coupling
``b`` uses ``T[group[b]]`` (or its transpose when ``transposed[b]``), so physical parameters (J shells,
DMI, anisotropic exchange) map onto ``T`` with ordinary torch operations and autograd applies the
chain rule.  ``A`` holds the per-sublattice single-ion tensors and ``B`` the external field.

The forward pass runs the trajectory in segments of ``seg_steps`` steps and keeps the spins at
segment starts (checkpoints).  The backward pass recomputes each segment from its checkpoint,
storing per step e, ep, both total fields and the two normalisation factors, then runs the adjoint
kernels (libmgx ``mgx_adjoint_*``) back through the segment.  The last segments that fit in
``cache_bytes`` keep their states from the forward pass and are not recomputed: checkpointing sized
to the memory one grants it ("auto", the default: half of the free device memory; 0: recompute every
segment).  Thermal (Philox) noise is regenerated bit-identically
from (seed, site, step), so the gradient is the pathwise derivative of the same noisy trajectory.
The forward and its recomputation run in the form GB300LLG's default would use for the system
(``precision="auto"``: the exact 56-bit fixed-point exchange sum on lattices where it is faster, FP64
otherwise); the adjoint kernels themselves are FP64.
magex itself has no gradients; parity of this module is pinned against central finite differences
and against torch autograd of a dense FP64 restatement (tests/test_gpu_adjoint.py).
"""
from __future__ import annotations

import copy
import ctypes as C

import numpy as np
import torch

from . import _lib
from .constants import GAMMA, K_B, MU_B
from .device import DeviceModel, stream_ptr
from .lattice import WIDTH_FULL
from .llg import _philox_key, auto_fixed


class CouplingGroups:
    """group[b], transposed[b] for every stencil coupling b, and the number of groups."""

    def __init__(self, group, transposed=None, ngroups=None):
        self.group = np.asarray(group, np.int32)
        self.transposed = np.zeros_like(self.group) if transposed is None else np.asarray(transposed, np.int32)
        self.ngroups = int(self.group.max()) + 1 if ngroups is None else int(ngroups)

    @classmethod
    def per_bond(cls, sc):
        """Every coupling its own tensor (dL/dJ_b for each coupling of the unit cell)."""
        return cls(np.arange(len(sc.bond_src)))

    @classmethod
    def symmetric_pairs(cls, sc):
        """One tensor per pair of mutually reverse couplings (i -> j, R) and (j -> i, -R) whose tensors
        are transposes of each other (J_ji = J_ij^T, true for every model built here): the reverse
        coupling uses the transposed group tensor.  Couplings without such a partner get their own
        group.  Half as many groups as per_bond, so half the gradient bookkeeping per site."""
        n = len(sc.bond_src)
        key = {(int(sc.bond_src[b]), int(sc.bond_dst[b]), tuple(int(x) for x in sc.bond_R[b])): b for b in range(n)}
        group = -np.ones(n, np.int32)
        trans = np.zeros(n, np.int32)
        g = 0
        for b in range(n):
            if group[b] >= 0:
                continue
            group[b] = g
            rb = key.get((int(sc.bond_dst[b]), int(sc.bond_src[b]), tuple(-int(x) for x in sc.bond_R[b])))
            if rb is not None and rb != b and group[rb] < 0 and np.array_equal(sc.bond_J[rb], sc.bond_J[b].T):
                group[rb] = g
                trans[rb] = 1
            g += 1
        return cls(group, trans, g)

    @classmethod
    def per_shell(cls, sc, ndigits=4):
        """One tensor per neighbour shell on canonical bonds (src < dst, or src == dst and R > 0) and its
        transpose on the reverse bonds: the shell-tensor parameterisation of the bcc workloads."""
        uc = sc.uc
        d = []
        for i, j, R in zip(sc.bond_src, sc.bond_dst, sc.bond_R):
            r = uc.positions[j] + R @ uc.cell - uc.positions[i]
            d.append(round(float(np.linalg.norm(r)), ndigits))
        shells = sorted(set(d))
        group = np.array([shells.index(x) for x in d], np.int32)
        trans = np.array([0 if (i < j or (i == j and tuple(R) > (0, 0, 0))) else 1
                          for i, j, R in zip(sc.bond_src, sc.bond_dst, sc.bond_R)], np.int32)
        return cls(group, trans, len(shells))

    def tensors_from(self, sc):
        """T (ngroups, 3, 3) consistent with the supercell's couplings (checked)."""
        T = np.zeros((self.ngroups, 3, 3))
        seen = np.zeros(self.ngroups, bool)
        for b, J in enumerate(sc.bond_J):
            g = self.group[b]
            Jg = J.T if self.transposed[b] else J
            if not seen[g]:
                T[g], seen[g] = Jg, True
            elif np.abs(T[g] - Jg).max() > 1e-12 * max(1.0, np.abs(Jg).max()):
                raise ValueError(f"coupling {b} does not match the tensor of its group {g}")
        return T

    def bond_tensors(self, T):
        """(nbond, 3, 3) coupling tensors of parameter tensors T (numpy)."""
        Tb = np.asarray(T, float)[self.group]
        return np.where(self.transposed[:, None, None] == 1, Tb.transpose(0, 2, 1), Tb)


def _full_width(sc):
    v = copy.copy(sc)
    v.width = WIDTH_FULL
    v.table = np.ascontiguousarray(sc.bond_J.reshape(-1, 9))
    return v


def _reverse(sc, groups):
    """Reverse stencil: coupling (j -> i, -R, J^T) for every forward (i -> j, R, J), ordered by receiving
    sublattice and then group; returns (view, order) with order[k] = forward bond of k."""
    order = sorted(range(len(sc.bond_src)), key=lambda b: (int(sc.bond_dst[b]), int(groups.group[b]), b))
    order = np.array(order, np.int64)
    v = copy.copy(sc)
    v.bond_src = np.ascontiguousarray(sc.bond_dst[order], np.int32)
    v.bond_dst = np.ascontiguousarray(sc.bond_src[order], np.int32)
    v.bond_R = np.ascontiguousarray(-sc.bond_R[order], np.int32)
    v.bond_J = np.ascontiguousarray(sc.bond_J[order].transpose(0, 2, 1))
    v.width = WIDTH_FULL
    v.table = np.ascontiguousarray(v.bond_J.reshape(-1, 9))
    return v, order


class AdjointLLG:
    """Forward / adjoint engine of Heun trajectories on one supercell (uniform alpha per run)."""

    def __init__(self, sc, groups=None, alpha=0.1, dt=1e-3, temperature=0.0, seed=None, precession=True,
                 seg_steps=100, cache_bytes="auto", precision="auto", device=None):
        if sc.alpha_site is not None or sc.site_T is not None or sc.A_site is not None:
            raise NotImplementedError("the adjoint supports uniform damping, temperature and per-sublattice A")
        if sc.terms or sc.has_higher:
            raise NotImplementedError("extra energy terms are not supported by the GB300 kernels")
        self.sc = sc
        self.groups = CouplingGroups.symmetric_pairs(sc) if groups is None else groups
        self.T0 = self.groups.tensors_from(sc)
        self.fwd = DeviceModel(_full_width(sc), device)
        rev_view, self.rev_order = _reverse(sc, self.groups)
        self.rev = DeviceModel(rev_view, device)
        self.device = self.fwd.device
        self.lib = self.fwd.lib
        self.alpha, self.dt, self.T = float(alpha), float(dt), float(temperature)
        self.seg_steps = int(seg_steps)
        p = _lib.LLGParams()
        p.dt, p.alpha, p.alpha_site = self.dt, self.alpha, None
        p.precession = int(bool(precession))
        p.integrator = _lib.HEUN
        p.noise = _lib.NOISE_PHILOX if self.T > 0 else _lib.NOISE_NONE
        p.seed = _philox_key(seed)
        # the forward (and its recomputation) in the form GB300LLG's default would step this system
        # with: the exact fixed-point exchange sum where "auto" picks it; the adjoint kernels are FP64
        if precision not in ("auto", "fp64", "fp64_fixed"):
            raise ValueError("precision must be 'auto', 'fp64' or 'fp64_fixed'")
        fixed = precision == "fp64_fixed" or (precision == "auto" and auto_fixed(sc, alpha))
        self.precision = "fp64_fixed" if fixed else "fp64"
        p.precision = _lib.PRECISION_FP64_FIXED_GATHER if fixed else _lib.PRECISION_FP64
        rg = np.ascontiguousarray(self.groups.group[self.rev_order], np.int32)
        rt = np.ascontiguousarray(self.groups.transposed[self.rev_order], np.int32)
        h = C.c_void_p()
        with torch.cuda.device(self.device):
            _lib.check(self.lib.mgx_adjoint_create(self.fwd.handle, self.rev.handle, _lib.iptr(rg), _lib.iptr(rt),
                                                   self.groups.ngroups, C.byref(p), self.seg_steps, C.byref(h)),
                       "mgx_adjoint_create")
        self.handle = h
        if self.T > 0:
            sig = np.ascontiguousarray(np.sqrt(2.0 * self.alpha * K_B * self.T / (GAMMA * sc.mu_sub * MU_B * self.dt)))
            _lib.check(self.lib.mgx_adjoint_set_sigma(h, _lib.dptr(sig)), "mgx_adjoint_set_sigma")
        ns, G = sc.ns, self.groups.ngroups
        self._grads = torch.empty(9 * G + 9 * ns + 3, dtype=torch.float64, device=self.device)
        self.storage_doubles = int(self.lib.mgx_adjoint_storage_doubles(h))
        if cache_bytes != "auto" and int(cache_bytes) < 0:
            raise ValueError("cache_bytes must be 'auto' or >= 0")
        self.cache_bytes = cache_bytes if cache_bytes == "auto" else int(cache_bytes)

    def _cache_budget(self):
        """Bytes of resident segment states: the given cache_bytes, or with "auto" half of the device
        memory free when the forward pass starts (GB300's HBM holds thousands of states of a 10^5-10^6
        spin lattice, so most trajectories run without any recomputation)."""
        if self.cache_bytes == "auto":
            free, _ = torch.cuda.mem_get_info(self.device)
            return int(0.5 * free)
        return self.cache_bytes

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            try:
                self.lib.mgx_adjoint_destroy(h)
            except Exception:
                pass
            self.handle = None

    # ------------------------------------------------------------------ parameters
    @property
    def has_higher(self):
        """The system carries cubic and / or higher-uniaxial anisotropy (magex/terms.py:35-75)."""
        return self.sc.cubic is not None or self.sc.uniaxial_higher is not None

    def set_higher(self, H):
        """Uniform cubic / higher-uniaxial constants H = (Kc, K2, K3) (meV) on every site of the forward
        model; the axes stay the system's.  Only the terms the system has are set."""
        Kc, K2, K3 = (float(x) for x in np.asarray(H, float).reshape(3))
        sc, N = self.sc, self.sc.N
        keep = []

        def arr(x):
            a = np.full(N, x, np.float64)
            keep.append(a)
            return _lib.dptr(a)
        cub, uni = sc.cubic, sc.uniaxial_higher
        Cm = None if cub is None else np.ascontiguousarray(np.asarray(cub[1], float).reshape(9))
        u = None if uni is None else np.ascontiguousarray(np.asarray(uni[2], float).reshape(3))
        _lib.check(self.lib.mgx_model_set_onsite_higher(
            self.fwd.handle, None if cub is None else arr(Kc), None if Cm is None else _lib.dptr(Cm),
            None if uni is None else arr(K2), None if uni is None else arr(K3), None if u is None else _lib.dptr(u)),
            "mgx_model_set_onsite_higher")
        _lib.check(self.lib.mgx_adjoint_sync_models(self.handle), "sync_models")

    def higher_params(self):
        """(Kc, K2, K3) of the system's first site (0 for absent terms)."""
        sc = self.sc
        Kc = 0.0 if sc.cubic is None else float(np.asarray(sc.cubic[0], float).reshape(-1)[0])
        K2 = 0.0 if sc.uniaxial_higher is None else float(np.asarray(sc.uniaxial_higher[0], float).reshape(-1)[0])
        K3 = 0.0 if sc.uniaxial_higher is None else float(np.asarray(sc.uniaxial_higher[1], float).reshape(-1)[0])
        return np.array([Kc, K2, K3])

    def set_params(self, T, A, B):
        """Load parameter tensors T (G,3,3), A (ns,3,3) and field B (3) into both device stencils."""
        T = np.asarray(T, float).reshape(self.groups.ngroups, 3, 3)
        Jf = np.ascontiguousarray(self.groups.bond_tensors(T).reshape(-1))
        Jr = np.ascontiguousarray(self.groups.bond_tensors(T)[self.rev_order].transpose(0, 2, 1).reshape(-1))
        A = np.ascontiguousarray(np.asarray(A, float).reshape(self.sc.ns, 9))
        _lib.check(self.lib.mgx_model_set_couplings(self.fwd.handle, _lib.dptr(Jf)), "set_couplings")
        _lib.check(self.lib.mgx_model_set_couplings(self.rev.handle, _lib.dptr(Jr)), "set_couplings")
        _lib.check(self.lib.mgx_model_set_onsite(self.fwd.handle, _lib.dptr(A)), "set_onsite")
        _lib.check(self.lib.mgx_model_set_onsite(self.rev.handle, _lib.dptr(A)), "set_onsite")
        Bv = (C.c_double * 3)(*[float(x) for x in np.asarray(B, float).reshape(3)])
        _lib.check(self.lib.mgx_model_set_field(self.fwd.handle, Bv), "set_field")
        self.fwd._B = np.array(list(Bv))
        self.fwd.sc.B = np.array(list(Bv))
        _lib.check(self.lib.mgx_adjoint_sync_models(self.handle), "sync_models")

    # ------------------------------------------------------------------ trajectory
    def _segments(self, nsteps):
        out, n = [], 0
        while n < nsteps:
            k = min(self.seg_steps, nsteps - n)
            out.append((n, k))
            n += k
        return out

    def forward(self, e0_lat, nsteps):
        """Run nsteps from lattice-layout spins; returns (e_T, checkpoints, resident segments).

        A checkpoint (the spins) is kept at the start of every segment of seg_steps steps.  When
        cache_bytes allows, the last segments also keep their full states (a resident segment costs
        mgx_adjoint_storage_doubles doubles), so the backward pass does not recompute them."""
        segs = self._segments(int(nsteps))
        ncache = min(len(segs), self._cache_budget() // (8 * self.storage_doubles))
        cache = [torch.empty(self.storage_doubles, dtype=torch.float64, device=self.device) for _ in range(ncache)]
        first_cached = len(segs) - ncache
        ckpts = []
        cur = e0_lat.contiguous()
        try:
            for k, (n0, m) in enumerate(segs):
                ckpts.append(cur)
                store = cache[k - first_cached] if k >= first_cached else None
                _lib.check(self.lib.mgx_adjoint_set_storage(self.handle, None if store is None else
                                                            C.c_void_p(store.data_ptr())), "set_storage")
                nxt = torch.empty_like(cur)
                _lib.check(self.lib.mgx_adjoint_forward(self.handle, C.c_void_p(cur.data_ptr()), m, n0,
                                                        C.c_void_p(nxt.data_ptr()), stream_ptr()), "mgx_adjoint_forward")
                cur = nxt
        finally:
            self.lib.mgx_adjoint_set_storage(self.handle, None)
        return cur, ckpts, cache

    def backward(self, ckpts, ebar_T_lat, nsteps, cache=(), needs=(True, True, True)):
        """dL/de_0 (lattice layout) and (dL/dT, dL/dA, dL/dB) from dL/de_T.  needs: which of the three
        parameter gradients to accumulate (the others come back as zeros)."""
        _lib.check(self.lib.mgx_adjoint_set_needs(self.handle, *(int(bool(x)) for x in needs)), "set_needs")
        ebar = ebar_T_lat.clone().contiguous()
        _lib.check(self.lib.mgx_adjoint_zero_grads(self.handle, stream_ptr()), "zero_grads")
        segs = self._segments(int(nsteps))
        first_cached = len(segs) - len(cache)
        # Segments without resident states are recomputed from their checkpoints into the plan's two
        # own storages, alternately, on a side stream: the recomputation of the next segment (earlier
        # in time) runs while the backward pass goes through the current one.  A storage is reused once
        # the backward pass through it has finished (event `free`), and a backward pass starts once its
        # segment is recomputed (event `ready`).
        main = torch.cuda.current_stream(self.device)
        if not hasattr(self, "_side"):
            self._side = torch.cuda.Stream(self.device)
        side = self._side
        free = [torch.cuda.Event(), torch.cuda.Event()]
        for ev in free:
            ev.record(main)
        pending = [k for k in range(len(segs) - 1, -1, -1) if k < first_cached]
        ready = {}

        def recompute(k):
            buf = k % 2
            side.wait_event(free[buf])
            _lib.check(self.lib.mgx_adjoint_select_own_storage(self.handle, buf), "select_own_storage")
            n0, m = segs[k]
            _lib.check(self.lib.mgx_adjoint_forward(self.handle, C.c_void_p(ckpts[k].data_ptr()), m, n0, None,
                                                    stream_ptr(side)), "mgx_adjoint_forward (recompute)")
            ready[k] = torch.cuda.Event()
            ready[k].record(side)

        nxt = 0
        if pending:
            recompute(pending[0])
            nxt = 1
        try:
            for k in range(len(segs) - 1, -1, -1):
                n0, m = segs[k]
                if k >= first_cached:
                    _lib.check(self.lib.mgx_adjoint_set_storage(self.handle, C.c_void_p(cache[k - first_cached].data_ptr())),
                               "set_storage")
                else:
                    main.wait_event(ready.pop(k))
                    if nxt < len(pending):
                        recompute(pending[nxt])
                        nxt += 1
                    _lib.check(self.lib.mgx_adjoint_select_own_storage(self.handle, k % 2), "select_own_storage")
                _lib.check(self.lib.mgx_adjoint_backward(self.handle, C.c_void_p(ebar.data_ptr()), m, stream_ptr(main)),
                           "mgx_adjoint_backward")
                if k < first_cached:
                    free[k % 2].record(main)
        finally:
            self.lib.mgx_adjoint_set_storage(self.handle, None)
            main.wait_stream(side)
        _lib.check(self.lib.mgx_adjoint_grads(self.handle, C.c_void_p(self._grads.data_ptr()), stream_ptr()),
                   "mgx_adjoint_grads")
        G, ns = self.groups.ngroups, self.sc.ns
        g = self._grads
        gT = g[:9 * G].view(G, 3, 3).clone()
        gA = g[9 * G:9 * G + 9 * ns].view(9, ns).t().reshape(ns, 3, 3).clone()
        gB = g[9 * G + 9 * ns:].clone()
        gH = torch.zeros(3, dtype=torch.float64, device=self.device)
        if self.has_higher:
            _lib.check(self.lib.mgx_adjoint_grads_onsite_higher(self.handle, C.c_void_p(gH.data_ptr()), stream_ptr()),
                       "mgx_adjoint_grads_onsite_higher")
        self.last_grad_higher = gH
        return ebar, gT, gA, gB


class _Trajectory(torch.autograd.Function):
    @staticmethod
    def forward(ctx, e0, T, A, B, H, adj, nsteps):
        params = (T.detach().cpu().numpy(), A.detach().cpu().numpy(), B.detach().cpu().numpy(),
                  None if H is None else H.detach().cpu().numpy())
        _Trajectory._load(adj, params)
        lat0 = adj.fwd.to_lattice(e0.detach())
        eT, ckpts, cache = adj.forward(lat0, nsteps)
        ctx.adj, ctx.nsteps, ctx.ckpts, ctx.cache = adj, nsteps, ckpts, cache
        ctx.devs = (e0.device, T.device, A.device, B.device, None if H is None else H.device)
        ctx.params = params
        out = adj.fwd.from_lattice(eT)
        return out.to(e0.device)

    @staticmethod
    def _load(adj, params):
        adj.set_params(*params[:3])
        if params[3] is not None:
            adj.set_higher(params[3])

    @staticmethod
    def backward(ctx, grad_eT):
        adj = ctx.adj
        _Trajectory._load(adj, ctx.params)           # the parameters may have changed since the forward
        ebar_T = adj.fwd.to_lattice(grad_eT.detach().contiguous())
        needs = ctx.needs_input_grad[1:4]            # T, A, B: accumulate only what autograd asks for
        ebar0, gT, gA, gB = adj.backward(ctx.ckpts, ebar_T, ctx.nsteps, ctx.cache, needs)
        ctx.cache = ()
        ge0 = adj.fwd.from_lattice(ebar0)
        d0, dT, dA, dB, dH = ctx.devs
        gH = None if dH is None else adj.last_grad_higher.to(dH)
        return (ge0.to(d0), gT.to(dT) if needs[0] else None, gA.to(dA) if needs[1] else None,
                gB.to(dB) if needs[2] else None, gH, None, None)


def llg_trajectory(adj, e0, T, A, B, nsteps, H=None):
    """Spins after nsteps Heun steps from e0 ((N,3) tensor), differentiable in e0, T, A and B, and in
    H = (Kc, K2, K3), uniform cubic / higher-uniaxial constants, when given (systems with those terms)."""
    if H is not None and not adj.has_higher:
        raise ValueError("H (Kc, K2, K3) needs a system with cubic or higher-uniaxial anisotropy")
    return _Trajectory.apply(e0, T, A, B, H, adj, int(nsteps))


_BOND_SITES: dict = {}


def bond_sites(sc, device):
    """Per stencil coupling b: (src, dst) magex site indices of every cell where it acts (cached)."""
    key = (id(sc), str(device))
    hit = _BOND_SITES.get(key)
    if hit is not None and hit[0] is sc:
        return hit[1]
    L = np.array(sc.L)
    c = np.stack(np.meshgrid(*[np.arange(n) for n in sc.L], indexing="ij"), -1).reshape(-1, 3)
    out = []
    for b in range(len(sc.bond_src)):
        t = c + sc.bond_R[b][None, :]
        ok = np.ones(len(c), bool)
        for a in range(3):
            if sc.pbc[a]:
                t[:, a] %= L[a]
            else:
                ok &= (t[:, a] >= 0) & (t[:, a] < L[a])
        cs, ts = c[ok], t[ok]
        src = ((cs[:, 0] * L[1] + cs[:, 1]) * L[2] + cs[:, 2]) * sc.ns + sc.bond_src[b]
        dst = ((ts[:, 0] * L[1] + ts[:, 1]) * L[2] + ts[:, 2]) * sc.ns + sc.bond_dst[b]
        out.append((torch.as_tensor(src, device=device), torch.as_tensor(dst, device=device)))
    _BOND_SITES.clear()
    _BOND_SITES[key] = (sc, out)
    return out


def energy_per_site(sc, groups, e, T, A, B):
    """Per-site energy (meV) of spins e ((N, 3), magex order) with the couplings of the parameter
    tensors T (ngroups, 3, 3), single-ion tensors A (ns, 3, 3) and field B (3,), differentiable in all
    four (torch autograd).  Terms as magex/spinmodel.py:475-484: -e.h - mu_B mu e.B + e A e, with
    h_i = sum_j J_ij e_j; their sum is the total energy, their mean the mean-energy loss."""
    dev, dt = e.device, e.dtype
    T = T.to(dev, dt)
    Tb = T[torch.as_tensor(groups.group, dtype=torch.long, device=dev)]
    tr = torch.as_tensor(groups.transposed, dtype=torch.bool, device=dev)[:, None, None]
    Jb = torch.where(tr, Tb.transpose(1, 2), Tb)
    h = torch.zeros_like(e)
    for b, (src, dst) in enumerate(bond_sites(sc, dev)):
        h = h.index_add(0, src, e[dst] @ Jb[b].T)
    As = A.to(dev, dt)[torch.as_tensor(sc.sublattice, dtype=torch.long, device=dev)]
    mu = torch.as_tensor(sc.mu, dtype=dt, device=dev)
    return torch.einsum("ia,iab,ib->i", e, As, e) - (e * h).sum(1) - MU_B * mu * (e @ B.to(dev, dt))
