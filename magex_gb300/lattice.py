"""Supercell description for the GB300 LLG kernels, built without the 3N x 3N sparse matrix.

magex builds every supercell as an explicit 3N x 3N CSR matrix (``magex/spinmodel.py:191-252``),
which needs O(N z 9) host memory and cannot be built at 10^7 - 10^8 spins.  On a periodic
(or open) Bravais supercell the couplings are translation invariant, so the whole exchange operator
is the per-cell coupling list itself: site (cell c, sublattice i) couples to site
(wrap(c + R), j) with tensor J for every coupling (i, j, R, J).  ``Supercell`` keeps exactly that
"stencil" (a few KB), and the CUDA kernels compute neighbour indices from it on the fly.

Site numbering follows magex: cells enumerate (c0, c1, c2) row-major and site = cell * ns + s
(``magex/spinmodel.py:197-204``).  The device layout (component-major, sublattice-major) is a
separate concern of ``magex_gb300.llg``.

Couplings that reach a site's own periodic image are single-site terms and are folded into the
single-ion tensor, A_i <- A_i - (J + J^T)/2, exactly as ``magex/spinmodel.py:224-229`` does.
"""
from __future__ import annotations

import itertools

import numpy as np

from .constants import MU_B
from .spinmodel import UnitCellModel, normalize

WIDTH_ISO, WIDTH_DMI, WIDTH_FULL = 1, 4, 9


def compress_tensors(tensors):
    """Choose the narrowest exact storage for a set of 3x3 coupling tensors.

    Returns (width, table) with table of shape (n, width):
      width 1: every tensor is J*I                      -> [J]
      width 4: every tensor is J*I + skew(D)            -> [J, Dx, Dy, Dz]  (J^A e = e x D)
      width 9: anything else                            -> row-major 3x3
    The tests are exact (no tolerance), so the compressed field equals the full product up to the
    order of the floating-point additions.  magex makes the same choice with a 1e-14 relative
    tolerance (``magex/fast.py:615-626``).
    """
    M = np.asarray(tensors, float).reshape(-1, 3, 3)
    if len(M) == 0:
        return WIDTH_ISO, np.zeros((0, 1))
    diag_equal = np.all(M[:, 0, 0] == M[:, 1, 1]) and np.all(M[:, 1, 1] == M[:, 2, 2])
    sym_off = M + M.transpose(0, 2, 1)
    antisym = np.all(sym_off[:, [0, 0, 1], [1, 2, 2]] == 0.0)
    if diag_equal and antisym:
        D = np.stack([M[:, 1, 2], M[:, 2, 0], M[:, 0, 1]], 1)
        if np.all(D == 0.0):
            return WIDTH_ISO, M[:, 0, 0][:, None].copy()
        return WIDTH_DMI, np.column_stack([M[:, 0, 0], D])
    return WIDTH_FULL, M.reshape(-1, 9).copy()


class _SpinTerms:
    """magex SpinSystem's energy terms for a lattice description (``N``, ``mu``): ``energy``,
    ``gradient`` and ``effective_field`` evaluated on the GPU, ``magnetization`` on the host.

    ``cubic = (Kc, C)`` (per-site Kc, 3x3 axes) and ``uniaxial_higher = (K2, K3, u)`` (per-site K2, K3,
    axis) are the cubic and higher uniaxial anisotropies of magex/terms.py:35-75 (None: absent).
    """

    cubic = None
    uniaxial_higher = None

    def magnetization(self, e, weighted=False):
        """Mean spin, or the moment-weighted mean (magex/spinmodel.py:521-524)."""
        e = np.asarray(e, float)
        return (self.mu[:, None] * e).sum(0) / self.mu.sum() if weighted else e.mean(0)

    # ------------------------------------------------------------------ energy terms, on the GPU
    def device_model(self):
        """The DeviceModel that ``energy`` / ``gradient`` / ``effective_field`` evaluate on, created
        on first use with the couplings and per-site terms of that moment; the external field follows
        ``set_field``."""
        dm = getattr(self, "_device_model", None)
        if dm is None:
            from .device import DeviceModel
            dm = self._device_model = DeviceModel(self)
        return dm

    def energy(self, e, per_spin=False):
        """Total energy (meV) of spins e ((N, 3), magex order), as magex/spinmodel.py:475-484."""
        dm = self.device_model()
        E = float(dm.observables(dm.to_lattice(e))[0].item())
        return E / self.N if per_spin else E

    def effective_field(self, e):
        """B_eff = -(dE/de) / (mu_B mu) in tesla, (N, 3) numpy (magex/spinmodel.py:471-473); zero
        on pinned sites."""
        dm = self.device_model()
        return dm.from_lattice(dm.effective_field(dm.to_lattice(e))).cpu().numpy()

    def gradient(self, e):
        """dE/de (meV), (N, 3) numpy (magex/spinmodel.py:458-469)."""
        return -MU_B * self.mu[:, None] * self.effective_field(e)


class Supercell(_SpinTerms):
    """Supercell of a UnitCellModel: the state the LLG kernels need, O(ns + couplings) in size.

    Mirrors the parts of magex ``SpinSystem`` that the LLG path reads (``N``, ``L``, ``pbc``,
    ``B`` / ``set_field``, ``mu``, ``A``, ``signs``, ``pinned``, ``site_T``, ``alpha_site``,
    ``positions``, ``sublattice``, ``init_spins``), with per-site arrays created lazily; per-site
    overrides (``A_site``, ``mu_site``, ``pinned``, ``site_T``, ``alpha_site``) may be assigned.
    ``energy``, ``gradient`` and ``effective_field`` are evaluated on the GPU; ``order_parameter``
    and ``magnetization`` on the host arrays, as magex computes them.
    """

    def __init__(self, uc: UnitCellModel, supercell=(10, 10, 10), pbc=(True, True, True),
                 field=(0.0, 0.0, 0.0)):
        self.uc = uc
        self.L = tuple(int(x) for x in supercell)
        self.pbc = tuple(bool(x) for x in pbc)
        if min(self.L) < 1:
            raise ValueError(f"supercell must be positive, got {self.L}")
        self.ns = uc.nsites
        self.ncell = int(np.prod(self.L))
        self.N = self.ncell * self.ns
        self.A_sub = np.array(uc.A, float).reshape(self.ns, 3, 3).copy()
        self.mu_sub = np.asarray(uc.moments, float).copy()
        self.signs_sub = np.asarray(uc.signs, float).copy()
        self.self_folded = 0
        src, dst, R, T = [], [], [], []
        for (i, j, Rv, Jt) in uc.couplings:
            Rv = np.asarray(Rv, int).reshape(3)
            Jt = np.asarray(Jt, float).reshape(3, 3)
            if self._reaches_own_image(i, j, Rv):
                self.A_sub[i] -= 0.5 * (Jt + Jt.T)
                self.self_folded += self.ncell
                continue
            src.append(i)
            dst.append(j)
            R.append(Rv)
            T.append(Jt)
        self.bond_src = np.array(src, np.int32)
        self.bond_dst = np.array(dst, np.int32)
        self.bond_R = np.array(R, np.int32).reshape(-1, 3)
        self.bond_J = np.array(T, float).reshape(-1, 3, 3)
        self.width, self.table = compress_tensors(self.bond_J)
        self.biquadratic = list(getattr(uc, "biquadratic", []) or [])
        self.four_spin = float(getattr(uc, "four_spin", 0.0) or 0.0)
        self.terms = []
        self.pinned = None
        self.pinned_dir = None
        self.site_T = None
        self.alpha_site = None
        self.A_site = None
        self.mu_site = None
        self.set_field(field)

    # ------------------------------------------------------------------ construction helpers
    def _reaches_own_image(self, i, j, R):
        if i != j:
            return False
        for a in range(3):
            if self.pbc[a]:
                if R[a] % self.L[a] != 0:
                    return False
            elif R[a] != 0:
                return False
        return True

    def set_field(self, B):
        self.B = np.asarray(B, float).reshape(3)

    # ------------------------------------------------------------------ per-site views (lazy)
    @property
    def sublattice(self):
        return np.tile(np.arange(self.ns), self.ncell)

    @property
    def cell_index(self):
        return np.repeat(np.arange(self.ncell), self.ns)

    @property
    def cells(self):
        return np.array(list(itertools.product(*[range(n) for n in self.L])), int)

    @property
    def positions(self):
        c = np.stack(np.meshgrid(*[np.arange(n) for n in self.L], indexing="ij"), -1).reshape(-1, 3)
        return (np.repeat(c, self.ns, 0) @ self.uc.cell) + np.tile(self.uc.positions, (self.ncell, 1))

    @property
    def mu(self):
        return self.mu_site if self.mu_site is not None else np.tile(self.mu_sub, self.ncell)

    @property
    def signs(self):
        return np.tile(self.signs_sub, self.ncell)

    @property
    def ref(self):
        return np.tile(np.asarray(self.uc.ref_dirs, float), (self.ncell, 1))

    @property
    def A(self):
        return self.A_site if self.A_site is not None else np.tile(self.A_sub, (self.ncell, 1, 1))

    @property
    def has_A(self):
        A = self.A_site if self.A_site is not None else self.A_sub
        return bool(np.max(np.abs(A)) > 0) if A.size else False

    @property
    def has_higher(self):
        return bool(self.biquadratic) or self.four_spin != 0.0

    # ------------------------------------------------------------------ spins
    def init_spins(self, kind="reference", axis=(0, 0, 1), seed=None, cone=0.0, path=None):
        """Initial spins as magex ``SpinSystem.init_spins`` (``magex/spinmodel.py:487-515``) for the
        kinds random / ferro / reference / reference_axis / file: same generator, same draws."""
        rng = np.random.default_rng(seed)
        if kind == "random":
            e = rng.normal(size=(self.N, 3))
        elif kind == "ferro":
            e = np.tile(np.asarray(axis, float), (self.N, 1))
        elif kind == "reference":
            e = self.ref.copy()
        elif kind == "reference_axis":
            ax = np.asarray(axis, float) / np.linalg.norm(axis)
            e = self.signs[:, None] * ax[None, :]
        elif kind == "file":
            e = np.load(path)["spins"] if str(path).endswith(".npz") else np.loadtxt(path, delimiter=",")[:, -3:]
            if e.shape != (self.N, 3):
                raise ValueError(f"spin file has shape {e.shape}, expected {(self.N, 3)}")
        else:
            raise ValueError(f"unknown initial state '{kind}' (textures are built by magex.structure)")
        if cone > 0:
            e = e + cone * rng.normal(size=e.shape)
        e = normalize(e)
        if self.pinned is not None and self.pinned_dir is not None:
            e[self.pinned] = self.pinned_dir[self.pinned]
        return e

    def order_parameter(self, e):
        """|sum_i s_i e_i| / N on host spins (magex ``magex/spinmodel.py:517-519``)."""
        return float(np.linalg.norm((self.signs[:, None] * e).sum(0)) / self.N)

    # ------------------------------------------------------------------ host CSR (reference order)
    def neighbour_csr(self):
        """Per-site neighbour list in magex site order: (ptr int64 (N+1), nbr int32, typ int32,
        table (ntypes, 9)).  Neighbours of a site are sorted by index and repeated (site, neighbour)
        pairs are merged into one summed tensor, which is the layout of ``magex/fast.py:587-627``.
        Used by the CPU restatement and by the arbitrary-lattice (CSR) device path."""
        ns, L, N = self.ns, np.array(self.L), self.N
        c = np.stack(np.meshgrid(*[np.arange(n) for n in self.L], indexing="ij"), -1).reshape(-1, 3)
        cidx = lambda q: (q[:, 0] * L[1] + q[:, 1]) * L[2] + q[:, 2]        # noqa: E731
        rows, cols, types = [], [], []
        for b in range(len(self.bond_src)):
            tgt = c + self.bond_R[b][None, :]
            ok = np.ones(self.ncell, bool)
            for a in range(3):
                if self.pbc[a]:
                    tgt[:, a] %= L[a]
                else:
                    ok &= (tgt[:, a] >= 0) & (tgt[:, a] < L[a])
            rows.append(cidx(c[ok]) * ns + self.bond_src[b])
            cols.append(cidx(tgt[ok]) * ns + self.bond_dst[b])
            types.append(np.full(int(ok.sum()), b, np.int64))
        if not rows:
            return np.zeros(N + 1, np.int64), np.zeros(0, np.int32), np.zeros(0, np.int32), np.zeros((1, 9))
        r = np.concatenate(rows).astype(np.int64)
        q = np.concatenate(cols).astype(np.int64)
        t = np.concatenate(types)
        order = np.lexsort((t, q, r))
        r, q, t = r[order], q[order], t[order]
        bondJ = self.bond_J.reshape(-1, 9)
        key = r * N + q
        first = np.ones(len(key), bool)
        first[1:] = key[1:] != key[:-1]
        if first.all():
            # no repeated pairs: the bond index is the table type
            uniq_J, inv = np.unique(bondJ, axis=0, return_inverse=True)
            typ = inv.reshape(-1)[t].astype(np.int32)
            table = uniq_J
            nbr = q.astype(np.int32)
            src = r
        else:
            grp = np.cumsum(first) - 1
            merged = np.zeros((int(grp[-1]) + 1, 9))
            np.add.at(merged, grp, bondJ[t])
            table, inv = np.unique(merged, axis=0, return_inverse=True)
            typ = inv.reshape(-1).astype(np.int32)
            nbr = q[first].astype(np.int32)
            src = r[first]
        ptr = np.zeros(N + 1, np.int64)
        np.add.at(ptr, src + 1, 1)
        return np.cumsum(ptr), nbr, typ, np.ascontiguousarray(table)

    def summary(self):
        return (f"GB300 supercell {self.L} pbc {self.pbc}: N = {self.N} spins, {self.ns} sublattices, "
                f"{len(self.bond_src)} stencil couplings (table width {self.width}), "
                f"B = {self.B.tolist()} T, mu_B = {MU_B}")


class NeighbourList(_SpinTerms):
    """Arbitrary spin system as per-site neighbour lists (carved shapes, vacancies, edited exchange).

    Built from a 3N x 3N coupling matrix the way magex builds its kernel tables
    (``magex/fast.py:587-627``): the 3x3 blocks of each (site, neighbour) pair, neighbours sorted by
    index, identical blocks stored once in a type table, compressed to width 1 / 4 when exact.  Carries
    the per-site arrays the LLG path reads; the device layout of its spins is magex's site order.
    """

    def __init__(self, ptr, nbr, typ, tensors, mu, A=None, signs=None, field=(0.0, 0.0, 0.0)):
        self.N = int(len(ptr) - 1)
        self.ns, self.ncell = 1, self.N
        self.L, self.pbc = (1, 1, self.N), (True, True, True)
        self.ptr = np.ascontiguousarray(ptr, np.int64)
        self.nbr = np.ascontiguousarray(nbr, np.int32)
        self.typ = np.ascontiguousarray(typ, np.int32)
        self.bond_J = np.asarray(tensors, float).reshape(-1, 3, 3)
        self.width, self.table = compress_tensors(self.bond_J)
        self.mu_site = np.ascontiguousarray(mu, float).reshape(self.N)
        self.mu_sub = np.ones(1)
        self.A_site = None if A is None else np.ascontiguousarray(A, float).reshape(self.N, 3, 3)
        self.A_sub = np.zeros((1, 3, 3))
        self.signs_site = np.ones(self.N) if signs is None else np.asarray(signs, float).reshape(self.N)
        self.signs_sub = np.ones(1)
        self.pinned = None
        self.pinned_dir = None
        self.site_T = None
        self.alpha_site = None
        self.terms = []
        self.biquadratic = []
        self.four_spin = 0.0
        self.set_field(field)

    @classmethod
    def from_matrix(cls, Jsp, mu, A=None, signs=None, field=(0.0, 0.0, 0.0)):
        """From a 3N x 3N (scipy) coupling matrix with J_ij in rows 3i..3i+2, columns 3j..3j+2."""
        J = Jsp.tocoo()
        N = J.shape[0] // 3
        i, j = J.row // 3, J.col // 3
        comp = 3 * (J.row % 3) + J.col % 3
        key = i.astype(np.int64) * N + j
        pairs, inv = np.unique(key, return_inverse=True)
        blocks = np.zeros((len(pairs), 9))
        np.add.at(blocks, (inv.reshape(-1), comp), J.data)
        src = pairs // N
        nbr = (pairs % N).astype(np.int32)
        ptr = np.zeros(N + 1, np.int64)
        np.add.at(ptr, src + 1, 1)
        tensors, typ = np.unique(blocks, axis=0, return_inverse=True) if len(blocks) else (np.zeros((0, 9)), np.zeros(0, int))
        return cls(np.cumsum(ptr), nbr, np.asarray(typ).reshape(-1), tensors, mu, A, signs, field)

    def set_field(self, B):
        self.B = np.asarray(B, float).reshape(3)

    @property
    def mu(self):
        return self.mu_site

    @property
    def signs(self):
        return self.signs_site

    @property
    def A(self):
        return self.A_site if self.A_site is not None else np.zeros((self.N, 3, 3))

    @property
    def has_A(self):
        return self.A_site is not None and bool(np.max(np.abs(self.A_site)) > 0)

    @property
    def has_higher(self):
        return False

    @property
    def sublattice(self):
        return np.zeros(self.N, int)

    def neighbour_csr(self):
        return self.ptr, self.nbr, self.typ, np.ascontiguousarray(self.bond_J.reshape(-1, 9))

    def order_parameter(self, e):
        return float(np.linalg.norm((self.signs[:, None] * e).sum(0)) / self.N)
