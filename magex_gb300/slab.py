"""Slab decomposition of one supercell along axis 0, with halo exchanges between the Heun stages.

This is the distributed single-lattice path of magex/mpi_spin.py:150-180: each rank owns a contiguous
range of c0 layers and keeps h halo layers on each side (h = the largest |R_0| of the couplings),
copies of its neighbours' boundary layers.  One Heun step is

    predictor on every local site  ->  exchange the halo layers of ep  ->
    corrector on every local site  ->  exchange the halo layers of e

so every owned site sees exactly the neighbours of the unsplit lattice.  Halo sites are stepped too
(their results are overwritten by the exchange), the Philox counters use the site index of the whole
lattice (``mgx_model_set_partition``), and observables sum only owned cells, so a split run equals the
unsplit one bit for bit.  Along axis 0 the local lattice is open: a periodic whole lattice gets its
wrap-around from the halos, an open one has no halo at its ends.

Transports move the packed halo layers (``mgx_lattice_layers``: one strided copy per message):
``LoopbackTransport`` between slabs held by one process (one GPU), ``DistTransport`` between ranks over
torch.distributed point-to-point (host-staged for gloo, device buffers for NCCL).
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib
from .device import stream_ptr
from .lattice import Supercell


def slab_ranges(L0, world):
    """Balanced contiguous c0 ranges [(start, stop)] of world slabs."""
    base, extra = divmod(int(L0), int(world))
    out, start = [], 0
    for r in range(world):
        n = base + (1 if r < extra else 0)
        out.append((start, start + n))
        start += n
    return out


def halo_depth(sc):
    """Largest |R_0| over the couplings of a Supercell (the halo depth along axis 0)."""
    R = np.asarray(sc.bond_R, int).reshape(-1, 3)
    return int(np.abs(R[:, 0]).max()) if len(R) else 0


class SlabGeometry:
    """Local extent, halo depths, owned layers and neighbours of slab `rank` of `world` along axis 0."""

    def __init__(self, L, pbc, h, world, rank):
        L = tuple(int(x) for x in L)
        if world < 1 or not 0 <= rank < world:
            raise ValueError(f"rank {rank} outside world of {world}")
        self.L, self.pbc, self.h, self.world, self.rank = L, tuple(bool(p) for p in pbc), int(h), world, rank
        self.start, self.stop = slab_ranges(L[0], world)[rank]
        nloc = self.stop - self.start
        periodic = self.pbc[0]
        split = world > 1 and self.h > 0
        if world > 1 and nloc < max(self.h, 1):
            raise ValueError(f"slab {rank} has {nloc} layers, fewer than the halo depth {self.h}")
        self.left_rank = (rank - 1) % world if split and (periodic or rank > 0) else None
        self.right_rank = (rank + 1) % world if split and (periodic or rank < world - 1) else None
        self.hl = self.h if self.left_rank is not None else 0
        self.hr = self.h if self.right_rank is not None else 0
        self.L_local = (nloc + self.hl + self.hr, L[1], L[2])
        self.pbc_local = (periodic if world == 1 else False, self.pbc[1], self.pbc[2])
        self.own = (self.hl, self.hl + nloc)
        self.cell_offset = (self.start - self.hl) * L[1] * L[2]

    def global_sites(self, ns):
        """magex site index in the whole lattice of every local site (local magex order)."""
        L0, L1, L2 = self.L
        c0 = (self.start - self.hl + np.arange(self.L_local[0])) % L0
        cells = ((c0[:, None] * L1 + np.arange(L1)[None, :])[:, :, None] * L2 + np.arange(L2)).reshape(-1)
        return (cells[:, None] * ns + np.arange(ns)[None, :]).reshape(-1)

    def owned_rows(self, ns):
        """Slice of the local magex-order rows that this slab owns (whole-lattice rows start*L1*L2*ns on)."""
        layer = self.L[1] * self.L[2] * ns
        return slice(self.own[0] * layer, self.own[1] * layer)


class SlabLLG:
    """One slab of a slab-decomposed GB300 LLG run (Philox noise; any precision form).

    Built from the unit-cell model and the whole lattice's size, boundaries and field; the solver is a
    GB300LLG on the local supercell (owned layers + halos) whose noise and observables are those of
    the whole lattice."""

    def __init__(self, uc, L, pbc, field, alpha, dt, temperature, seed, rank, world, precession=True,
                 integrator="heun", precision="fp64", device=None):
        from .llg import GB300LLG
        whole = Supercell(uc, L, pbc, field)
        self.geo = SlabGeometry(L, pbc, halo_depth(whole), world, rank)
        self.sc = Supercell(uc, self.geo.L_local, self.geo.pbc_local, field)
        self.solver = GB300LLG(self.sc, alpha, dt, temperature, seed, precession=precession, integrator=integrator,
                               precision=precision, device=device)
        self.model = self.solver.model
        self.lib = _lib.load()
        _lib.check(self.lib.mgx_model_set_partition(self.model.handle, self.geo.cell_offset, *self.geo.own),
                   "mgx_model_set_partition")
        ptr = C.c_void_p()
        _lib.check(self.lib.mgx_llg_predicted(self.solver.handle, C.byref(ptr)), "mgx_llg_predicted")
        self._ep = ptr
        eps = C.c_void_p()
        _lib.check(self.lib.mgx_llg_predicted_split(self.solver.handle, C.byref(eps)), "mgx_llg_predicted_split")
        self._eps = eps if eps.value else None      # split copy of ep the reduced / fixed-point forms gather from
        self._layer = 3 * self.sc.ns * self.sc.L[1] * self.sc.L[2]
        self._sites = self.geo.global_sites(self.sc.ns)

    # ------------------------------------------------------------------ data movement
    def scatter(self, e_whole):
        """Local lattice-layout spins (owned + halo layers) from the whole lattice's (N, 3) spins."""
        return self.model.to_lattice(np.asarray(e_whole, np.float64)[self._sites])

    def owned(self, lat):
        """(N_owned, 3) numpy spins of the owned layers (rows start*L1*L2*ns ... of the whole lattice)."""
        return self.model.from_lattice(lat).cpu().numpy()[self.geo.owned_rows(self.sc.ns)]

    def _ptr(self, which, lat):
        if which == "eps":
            return self._eps
        return self._ep if which == "ep" else C.c_void_p(lat.data_ptr())

    def _fields(self, which):
        """Arrays exchanged for a halo message: ep travels with its split copy (8-byte elements too)."""
        return ("ep", "eps") if which == "ep" and self._eps is not None else (which,)

    def _layers(self, which, lat, c0a, c0b, buf, to_buffer, stream=None):
        _lib.check(self.lib.mgx_lattice_layers(self.model.handle, self._ptr(which, lat), c0a, c0b,
                                               C.c_void_p(buf.data_ptr()), int(to_buffer), stream_ptr(stream)),
                   "mgx_lattice_layers")

    def pack(self, which, lat):
        """Boundary layers to send: the first h owned layers to the left neighbour, the last h to the right
        (one message per side, the exchanged arrays one after the other)."""
        g, out = self.geo, {}
        a, b = g.own
        fields = self._fields(which)
        n = self._layer * g.h
        for side, lo in (("left", a), ("right", b - g.h)):
            if (g.left_rank if side == "left" else g.right_rank) is None:
                continue
            buf = torch.empty(n * len(fields), dtype=torch.float64, device=lat.device)
            for k, f in enumerate(fields):
                self._layers(f, lat, lo, lo + g.h, buf[k * n:(k + 1) * n], True)
            out[side] = buf
        return out

    def unpack(self, which, lat, recv):
        """Received halo layers into layers [0, hl) and [own_end, own_end + hr)."""
        g = self.geo
        fields = self._fields(which)
        for side, lo, depth in (("left", 0, g.hl), ("right", g.own[1], g.hr)):
            if side not in recv:
                continue
            buf = recv[side].to(lat.device)
            n = self._layer * depth
            for k, f in enumerate(fields):
                self._layers(f, lat, lo, lo + depth, buf[k * n:(k + 1) * n], False)

    # ------------------------------------------------------------------ stages and observables
    def stage(self, lat, k):
        self.solver.stage_lattice(lat, k)

    def observables(self, lat):
        """Partial [E, sum e (3), sum s e (3), max torque] over the owned cells (float64 numpy)."""
        return self.model.observables(lat).cpu().numpy().copy()


class LoopbackTransport:
    """Halo exchange between slabs held by one process: the receiver copies the sender's buffer."""

    def exchange(self, slabs, sends):
        by_rank = {sl.geo.rank: s for sl, s in zip(slabs, sends)}
        recvs = []
        for sl in slabs:
            g, r = sl.geo, {}
            if g.left_rank is not None:
                r["left"] = by_rank[g.left_rank]["right"]
            if g.right_rank is not None:
                r["right"] = by_rank[g.right_rank]["left"]
            recvs.append(r)
        return recvs

    def reduce(self, parts):
        out = np.sum([p[:7] for p in parts], axis=0)
        return np.concatenate([out, [max(p[7] for p in parts)]])


class DistTransport:
    """Halo exchange between ranks (one slab each) over torch.distributed point-to-point messages:
    tag 0 travels to the left neighbour, tag 1 to the right.  Buffers are staged through host memory
    for the gloo backend."""

    def __init__(self, group=None):
        import torch.distributed as dist
        self.dist = dist
        self.group = group
        self.host = dist.get_backend(group) == "gloo"

    def _stage(self, t):
        return t.cpu() if self.host else t

    def exchange(self, slabs, sends):
        (sl,) = slabs
        (send,) = sends
        g, d = sl.geo, self.dist
        recv, ops = {}, []
        if g.left_rank is not None:
            recv["left"] = torch.empty_like(self._stage(send["left"]))
            ops.append(d.P2POp(d.isend, self._stage(send["left"]), g.left_rank, self.group, 0))
            ops.append(d.P2POp(d.irecv, recv["left"], g.left_rank, self.group, 1))
        if g.right_rank is not None:
            recv["right"] = torch.empty_like(self._stage(send["right"]))
            ops.append(d.P2POp(d.isend, self._stage(send["right"]), g.right_rank, self.group, 1))
            ops.append(d.P2POp(d.irecv, recv["right"], g.right_rank, self.group, 0))
        if ops:
            for req in d.batch_isend_irecv(ops):
                req.wait()
        return [recv]

    def reduce(self, parts):
        (p,) = parts
        t = torch.as_tensor(np.asarray(p[:7], np.float64))
        m = torch.as_tensor(np.asarray(p[7:8], np.float64))
        self.dist.all_reduce(t, group=self.group)
        self.dist.all_reduce(m, op=self.dist.ReduceOp.MAX, group=self.group)
        return np.concatenate([t.numpy(), m.numpy()])


class SlabRun:
    """Heun steps of the slabs held by this process, exchanging halos through `transport`."""

    def __init__(self, slabs, transport):
        self.slabs = list(slabs)
        self.transport = transport

    def exchange(self, which, lats):
        sends = [sl.pack(which, lat) for sl, lat in zip(self.slabs, lats)]
        recvs = self.transport.exchange(self.slabs, sends)
        for sl, lat, r in zip(self.slabs, lats, recvs):
            sl.unpack(which, lat, r)

    def step(self, lats):
        for sl, lat in zip(self.slabs, lats):
            sl.stage(lat, 0)
        self.exchange("ep", lats)
        for sl, lat in zip(self.slabs, lats):
            sl.stage(lat, 1)
        self.exchange("e", lats)

    def run(self, lats, nsteps):
        for _ in range(int(nsteps)):
            self.step(lats)

    def observables(self, lats):
        """[E, sum e (3), sum s e (3), max torque] of the whole lattice."""
        return self.transport.reduce([sl.observables(lat) for sl, lat in zip(self.slabs, lats)])
