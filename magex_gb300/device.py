"""Device-resident model: a Supercell uploaded to the GB300 through the C ABI (mgx_model_*).

``DeviceModel`` owns one ``mgx_model`` handle and offers the layout conversions and observables
that the LLG driver needs.  Spins live on the device in the lattice layout (a (3, N) float64
tensor, component-major, sublattice-major); magex's (N, 3) arrays are converted at the boundary.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib
from .lattice import NeighbourList, Supercell


def _require_cuda():
    if not torch.cuda.is_available():
        raise RuntimeError("the GB300 LLG path needs a CUDA device (there is no CPU fallback)")


def stream_ptr(stream=None):
    s = torch.cuda.current_stream() if stream is None else stream
    return C.c_void_p(s.cuda_stream)


def supercell_from_system(system):
    """Supercell for a magex ``SpinSystem`` (or a Supercell, returned as is).

    The coupling stencil is rebuilt from ``system.uc`` and checked against ``system.Jsp`` so that a
    system whose exchange was edited after construction (carving, interface scaling) is refused
    instead of being integrated with the wrong couplings.  Per-site single-ion tensors, moments,
    pinning, site temperatures and damping set by ``magex.structure`` are carried over, and so are the
    first cubic and higher uniaxial anisotropy terms (the on-site terms of magex's fused kernels).  Terms
    the kernels do not implement (biquadratic, four-spin, dipolar, quadruplets) raise
    NotImplementedError, as ``magex/cuda_backend.py:315-316`` does.
    """
    if isinstance(system, (Supercell, NeighbourList)):
        sc = system
    else:
        if getattr(system, "has_higher", False):
            raise NotImplementedError("biquadratic / four-spin couplings are not supported by the GB300 kernels")
        sc = Supercell(system.uc, system.L, system.pbc, getattr(system, "B", (0.0, 0.0, 0.0)))
        Jsp = getattr(system, "Jsp", None)
        if int(system.N) != sc.N or (Jsp is not None and not _stencil_matches(sc, Jsp)):
            # carved or edited: the per-site neighbour-list layout
            sc = NeighbourList.from_matrix(Jsp, np.asarray(system.mu, float), np.asarray(system.A, float),
                                           np.asarray(system.signs, float), getattr(system, "B", (0.0, 0.0, 0.0)))
            for name in ("pinned", "pinned_dir", "site_T", "alpha_site"):
                v = getattr(system, name, None)
                if v is not None:
                    setattr(sc, name, np.array(v))
            _take_onsite_terms(sc, getattr(system, "terms", []))
            return sc
        A = np.asarray(system.A, float).reshape(sc.N, 3, 3)
        if not np.array_equal(A, np.tile(sc.A_sub, (sc.ncell, 1, 1))):
            sc.A_site = A.copy()
        mu = np.asarray(system.mu, float).reshape(sc.N)
        if not np.array_equal(mu, np.tile(sc.mu_sub, sc.ncell)):
            sc.mu_site = mu.copy()
        for name in ("pinned", "pinned_dir", "site_T", "alpha_site"):
            v = getattr(system, name, None)
            if v is not None:
                setattr(sc, name, np.array(v))
        _take_onsite_terms(sc, getattr(system, "terms", []))
    if getattr(sc, "terms", None):
        raise NotImplementedError("extra energy terms (dipolar, quadruplets) are not supported by the GB300 kernels")
    if sc.has_higher:
        raise NotImplementedError("biquadratic / four-spin couplings are not supported by the GB300 kernels")
    return sc


def _take_onsite_terms(sc, terms):
    """The first cubic (Kc, C) and the first higher uniaxial (K2, K3, u) term of a magex system go to the
    kernels, as magex/fast.py:647-652 splits them off; anything else (dipolar, quadruplets, a second
    term of either kind) raises NotImplementedError, as magex/cuda_backend.py:315-316 does."""
    rest = []
    for t in terms or []:
        kind = type(t).__name__
        if kind == "CubicAnisotropy" and getattr(sc, "cubic", None) is None:
            sc.cubic = (np.array(t.Kc, float), np.array(t.C, float))
        elif kind == "UniaxialHigher" and getattr(sc, "uniaxial_higher", None) is None:
            sc.uniaxial_higher = (np.array(t.K2, float), np.array(t.K3, float), np.array(t.u, float))
        else:
            rest.append(t)
    sc.terms = []
    if rest:
        raise NotImplementedError("extra energy terms (dipolar, quadruplets) are not supported by the GB300 kernels")


def _stencil_matches(sc, Jsp):
    """True when the stencil reproduces the system's sparse coupling matrix (same non-zeros and values)."""
    import scipy.sparse as sp
    ptr, nbr, typ, table = sc.neighbour_csr()
    N = sc.N
    rows = np.repeat(np.arange(N), np.diff(ptr))
    blocks = table[typ].reshape(-1, 3, 3)
    a, b = np.meshgrid(np.arange(3), np.arange(3), indexing="ij")
    R = (3 * rows[:, None, None] + a[None]).ravel()
    Cc = (3 * nbr.astype(np.int64)[:, None, None] + b[None]).ravel()
    mine = sp.csr_matrix((blocks.ravel(), (R, Cc)), shape=(3 * N, 3 * N))
    diff = abs(Jsp.tocsr() - mine)
    scale = max(float(abs(Jsp).max()) if Jsp.nnz else 0.0, 1e-300)
    return not (diff.nnz and float(diff.max()) > 1e-12 * scale)


def stencil_desc(sc):
    """mgx_lattice_desc of a Supercell and the host arrays it points into (keep them alive)."""
    d = _lib.LatticeDesc()
    d.ns = sc.ns
    d.L[:] = list(sc.L)
    d.pbc[:] = [int(p) for p in sc.pbc]
    d.nbond = len(sc.bond_src)
    src = np.ascontiguousarray(sc.bond_src, np.int32)
    dst = np.ascontiguousarray(sc.bond_dst, np.int32)
    R = np.ascontiguousarray(sc.bond_R, np.int32).reshape(-1)
    tab = np.ascontiguousarray(sc.table, np.float64).reshape(-1)
    A = np.ascontiguousarray(sc.A_sub, np.float64).reshape(-1)
    mu = np.ascontiguousarray(sc.mu_sub, np.float64)
    sg = np.ascontiguousarray(sc.signs_sub, np.float64)
    d.bond_src, d.bond_dst, d.bond_R = _lib.iptr(src), _lib.iptr(dst), _lib.iptr(R)
    d.width = sc.width
    d.bond_table = _lib.dptr(tab)
    d.A_sub = _lib.dptr(A)
    d.mu_sub = _lib.dptr(mu)
    d.sign_sub = _lib.dptr(sg)
    d.B[:] = [float(x) for x in sc.B]
    return d, [src, dst, R, tab, A, mu, sg]


class DeviceModel:
    """An ``mgx_model`` on the current CUDA device built from a Supercell."""

    def __init__(self, sc: Supercell, device=None):
        _require_cuda()
        self.lib = _lib.load()
        self.sc = sc
        self.device = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
        self.N = sc.N
        self._keep = []
        if isinstance(sc, NeighbourList):
            self._create_csr(sc)
            self._set_higher_onsite(sc)
            return
        nb = len(sc.bond_src)
        if nb > _lib.MAX_BONDS:
            raise NotImplementedError(f"{nb} couplings per cell exceed the kernel limit of {_lib.MAX_BONDS}")
        if sc.ns > _lib.MAX_SUBLATTICES:
            raise NotImplementedError(f"{sc.ns} sublattices exceed the kernel limit of {_lib.MAX_SUBLATTICES}")
        d, self._keep = stencil_desc(sc)
        sites = _lib.SiteDesc()
        if sc.A_site is not None:
            a = np.ascontiguousarray(sc.A_site, np.float64).reshape(-1)
            self._keep.append(a)
            sites.A_site = _lib.dptr(a)
        if sc.mu_site is not None:
            m = np.ascontiguousarray(sc.mu_site, np.float64)
            self._keep.append(m)
            sites.mu_site = _lib.dptr(m)
        if sc.pinned is not None:
            p = np.ascontiguousarray(np.asarray(sc.pinned, bool), np.uint8)
            self._keep.append(p)
            sites.pinned = _lib.u8ptr(p)
        h = C.c_void_p()
        with torch.cuda.device(self.device):
            _lib.check(self.lib.mgx_model_create(C.byref(d), C.byref(sites), C.byref(h)), "mgx_model_create")
        self.handle = h
        self._keep = []
        self._B = np.array(sc.B, float)
        self._obs = torch.empty(8, dtype=torch.float64, device=self.device)
        self._tri = None
        self.field_owner = None
        self._set_higher_onsite(sc)

    def _set_higher_onsite(self, sc):
        """Cubic and higher uniaxial anisotropy of the lattice (mgx_model_set_onsite_higher)."""
        cub, uni = getattr(sc, "cubic", None), getattr(sc, "uniaxial_higher", None)
        if cub is None and uni is None:
            return
        N = sc.N
        arr = lambda x, n: np.ascontiguousarray(np.broadcast_to(np.asarray(x, float), (n,)), np.float64)  # noqa: E731
        Kc = Cm = K2 = K3 = u = None
        if cub is not None:
            Kc, Cm = arr(cub[0], N), np.ascontiguousarray(np.asarray(cub[1], float).reshape(9))
        if uni is not None:
            K2, K3, u = arr(uni[0], N), arr(uni[1], N), np.ascontiguousarray(np.asarray(uni[2], float).reshape(3))
        p = lambda a: None if a is None else _lib.dptr(a)                                              # noqa: E731
        with torch.cuda.device(self.device):
            _lib.check(self.lib.mgx_model_set_onsite_higher(self.handle, p(Kc), p(Cm), p(K2), p(K3), p(u)),
                       "mgx_model_set_onsite_higher")

    def _create_csr(self, sc):
        c = _lib.CSRDesc()
        c.nsites = sc.N
        ptr = np.ascontiguousarray(sc.ptr, np.int64)
        nbr = np.ascontiguousarray(sc.nbr, np.int32)
        typ = np.ascontiguousarray(sc.typ, np.int32)
        tab = np.ascontiguousarray(sc.table, np.float64).reshape(-1)
        mu = np.ascontiguousarray(sc.mu_site, np.float64)
        sg = np.ascontiguousarray(sc.signs_site, np.float64)
        A = None if sc.A_site is None else np.ascontiguousarray(sc.A_site, np.float64).reshape(-1)
        pin = None if sc.pinned is None else np.ascontiguousarray(np.asarray(sc.pinned, bool), np.uint8)
        keep = [ptr, nbr, typ, tab, mu, sg, A, pin]
        c.ptr = ptr.ctypes.data_as(C.POINTER(C.c_int64))
        c.nbr, c.typ = _lib.iptr(nbr), _lib.iptr(typ)
        c.ntypes = len(sc.table)
        c.width = sc.width
        c.table = _lib.dptr(tab)
        c.A_site = _lib.dptr(A)
        c.mu_site = _lib.dptr(mu)
        c.sign_site = _lib.dptr(sg)
        c.pinned = _lib.u8ptr(pin)
        c.B[:] = [float(x) for x in sc.B]
        h = C.c_void_p()
        with torch.cuda.device(self.device):
            _lib.check(self.lib.mgx_model_create_csr(C.byref(c), C.byref(h)), "mgx_model_create_csr")
        del keep
        self.handle = h
        self._B = np.array(sc.B, float)
        self._obs = torch.empty(8, dtype=torch.float64, device=self.device)
        self._tri = None
        self.field_owner = None

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            try:
                self.lib.mgx_model_destroy(h)
            except Exception:
                pass
            self.handle = None

    # ------------------------------------------------------------------ state sync
    def sync_field(self):
        """Push a changed external field (SpinSystem.set_field) to the device model.  The field is
        read from ``field_owner`` (the magex SpinSystem a solver was built from) when set."""
        owner = self.field_owner if self.field_owner is not None else self.sc
        B = np.asarray(owner.B, float).reshape(3)
        if not np.array_equal(B, self._B):
            arr = (C.c_double * 3)(*[float(x) for x in B])
            _lib.check(self.lib.mgx_model_set_field(self.handle, arr), "mgx_model_set_field")
            self._B = B.copy()

    def push_field(self, B):
        """Set the device model's external field to B (T) now; sync_field restores the owner's field
        when that differs."""
        B = np.asarray(B, float).reshape(3)
        arr = (C.c_double * 3)(*[float(x) for x in B])
        _lib.check(self.lib.mgx_model_set_field(self.handle, arr), "mgx_model_set_field")
        self._B = B.copy()

    # ------------------------------------------------------------------ layout
    def to_lattice(self, e, out=None, stream=None):
        """(N, 3) spins (numpy or torch, any device) -> (3, N) float64 lattice-layout tensor."""
        src = torch.as_tensor(e, dtype=torch.float64)
        if src.shape != (self.N, 3):
            raise ValueError(f"spins have shape {tuple(src.shape)}, expected {(self.N, 3)}")
        src = src.to(self.device, non_blocking=True).contiguous()
        out = torch.empty((3, self.N), dtype=torch.float64, device=self.device) if out is None else out
        _lib.check(self.lib.mgx_pack_spins(self.handle, C.c_void_p(src.data_ptr()), C.c_void_p(out.data_ptr()),
                                           stream_ptr(stream)), "mgx_pack_spins")
        return out

    def from_lattice(self, lat, out=None, stream=None):
        """(3, N) lattice-layout tensor -> (N, 3) device tensor in magex site order."""
        out = torch.empty((self.N, 3), dtype=torch.float64, device=self.device) if out is None else out
        _lib.check(self.lib.mgx_unpack_spins(self.handle, C.c_void_p(lat.data_ptr()), C.c_void_p(out.data_ptr()),
                                             stream_ptr(stream)), "mgx_unpack_spins")
        return out

    # ------------------------------------------------------------------ observables
    def observables(self, lat, stream=None):
        """Device tensor [E, sum e (3), sum s e (3), max |e x B_eff|] of lattice-layout spins."""
        self.sync_field()
        _lib.check(self.lib.mgx_observables(self.handle, C.c_void_p(lat.data_ptr()), C.c_void_p(self._obs.data_ptr()),
                                            stream_ptr(stream)), "mgx_observables")
        return self._obs

    def effective_field(self, lat, stream=None):
        self.sync_field()
        B = torch.empty_like(lat)
        _lib.check(self.lib.mgx_effective_field(self.handle, C.c_void_p(lat.data_ptr()), C.c_void_p(B.data_ptr()),
                                                stream_ptr(stream)), "mgx_effective_field")
        return B

    def set_triangles(self, tri_sites, orient):
        """Triangle list (magex site indices, (T, 3)) and orientation signs for topological charge."""
        sc = self.sc
        tri = np.asarray(tri_sites, np.int64).reshape(-1, 3)
        if tri.size and (tri.min() < 0 or tri.max() >= sc.N):
            raise ValueError("triangle vertices must be site indices in [0, N)")
        if len(np.asarray(orient).reshape(-1)) != len(tri):
            raise ValueError("one orientation sign per triangle")
        cell, s = tri // sc.ns, tri % sc.ns
        lat_idx = (s * sc.ncell + cell).astype(np.int32)
        self._tri = torch.as_tensor(np.ascontiguousarray(lat_idx.reshape(-1)), device=self.device)
        self._orient = torch.as_tensor(np.ascontiguousarray(orient, np.float64), device=self.device)
        self._Q = torch.empty(1, dtype=torch.float64, device=self.device)

    def topological_charge(self, lat, stream=None):
        if self._tri is None:
            raise RuntimeError("set_triangles() first")
        _lib.check(self.lib.mgx_topological_charge(
            self.handle, C.c_void_p(lat.data_ptr()), C.c_void_p(self._tri.data_ptr()),
            C.c_void_p(self._orient.data_ptr()), C.c_int64(self._orient.numel()), C.c_void_p(self._Q.data_ptr()),
            stream_ptr(stream)), "mgx_topological_charge")
        return self._Q
