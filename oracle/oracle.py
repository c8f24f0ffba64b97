"""Python side of the CPU oracle (liboracle.so, built from oracle/heun_ref.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
leg, never by the magex_gb300 package.

``OracleLLG`` restates magex's LLG step on the CPU: the Heun / Depondt predictor-corrector of
magex/fast.py:336-390 (operation order of the reference's fused kernels, which it shows to agree
with the NumPy path magex/llg.py:216-227 to 1e-12), the thermal amplitude of magex/llg.py:106-122
and the observables of magex/spinmodel.py:475-484,517-519 and magex/llg.py:250-252,265.

Noise modes: "host" draws ``numpy.random.default_rng(seed).normal(size=(N, 3))`` per step exactly
like magex's NumPy path; "ziggurat" ports magex's numba generator (xorshift64* + ziggurat,
magex/fast.py:123-200,683-688), used to time the CPU baseline.

Parity of this oracle with the reference is pinned by tests/test_oracle_golden.py against
trajectories generated by the reference itself (tests/golden/make_golden.py).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
# the same source built at -O3 with host-CPU tuning: only the CPU-baseline timing loads it
LIB_TUNED = os.path.join(HERE, "liboracle_tuned.so")
MU_B = 5.7883818060e-2
K_B = 8.617333262e-2
GAMMA = 0.1760859630

_dp = C.POINTER(C.c_double)


class _Model(C.Structure):
    _fields_ = [("N", C.c_int64), ("ptr", C.POINTER(C.c_int64)), ("nbr", C.POINTER(C.c_int32)),
                ("typ", C.POINTER(C.c_int32)), ("table", _dp), ("width", C.c_int32), ("A", _dp), ("mu", _dp),
                ("B", C.c_double * 3), ("pinned", C.POINTER(C.c_uint8)),
                ("Kc", _dp), ("C", C.c_double * 9), ("K2", _dp), ("K3", _dp), ("u", C.c_double * 3)]


_lib = None


def build(force=False):
    """Compile liboracle.so and liboracle_tuned.so with the Makefile next to this file (gcc, OpenMP)."""
    src = os.path.getmtime(os.path.join(HERE, "heun_ref.c"))
    if force or any(not os.path.exists(p) or os.path.getmtime(p) < src for p in (LIB, LIB_TUNED)):
        r = subprocess.run(["make", "-C", HERE, "-B" if force else "all"], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    return LIB


def tuned_flags():
    """Compiler flags of liboracle_tuned.so (recorded by the Makefile when it built the library)."""
    build()
    with open(os.path.join(HERE, "liboracle_tuned.flags")) as f:
        return f.read().strip()


_lib_tuned = None


def load(tuned=False):
    """The parity oracle (liboracle.so), or with tuned=True its -O3 host-tuned build for timing."""
    global _lib, _lib_tuned
    if tuned:
        if _lib_tuned is None:
            build()
            _lib_tuned = _bind(C.CDLL(LIB_TUNED))
        return _lib_tuned
    if _lib is None:
        build()
        _lib = _bind(C.CDLL(LIB))
    return _lib


def _bind(lib):
    """Argument and result types of the oracle's exported functions."""
    lib.oracle_step.argtypes = [C.POINTER(_Model), _dp, C.c_double, C.c_int, C.c_int, _dp, _dp, _dp, _dp, C.c_int]
    lib.oracle_step.restype = None
    lib.oracle_stage.argtypes = [C.POINTER(_Model), _dp, C.c_double, C.c_int, C.c_int, _dp, _dp, _dp, _dp, C.c_int,
                                 C.c_int]
    lib.oracle_stage.restype = None
    lib.oracle_observables.argtypes = [C.POINTER(_Model), _dp, _dp, _dp, C.c_int]
    lib.oracle_observables.restype = None
    lib.oracle_gauss3.argtypes = [_dp, C.POINTER(C.c_uint64), C.c_int, _dp, C.POINTER(C.c_uint8), C.c_int64, C.c_int]
    lib.oracle_gauss3.restype = None
    lib.oracle_max_threads.restype = C.c_int
    ip = C.POINTER(C.c_int32)
    lib.oracle_stencil_csr.argtypes = [C.c_int, ip, ip, C.c_int, ip, ip, ip, ip, C.POINTER(C.c_int64), ip, ip]
    lib.oracle_stencil_csr.restype = C.c_int64
    lib.oracle_greedy_colour.argtypes = [C.c_int64, C.POINTER(C.c_int64), ip, ip]
    lib.oracle_greedy_colour.restype = C.c_int32
    lib.oracle_mc_group.argtypes = [C.POINTER(_Model), C.POINTER(C.c_int64), C.c_int64, C.c_int, _dp, C.c_double,
                                    _dp, _dp, C.c_int]
    lib.oracle_mc_group.restype = C.c_int64
    return lib


def max_threads():
    return int(load().oracle_max_threads())


def _p(a, t=_dp):
    return None if a is None else a.ctypes.data_as(t)


def stencil_csr(sc):
    """magex-order per-site neighbour list of a Supercell built by the C helper (fast at 10^6-10^7
    sites).  Every stencil coupling is its own table type; neighbours keep the coupling order."""
    lib = load()
    ip = C.POINTER(C.c_int32)
    L = np.array(sc.L, np.int32)
    pbc = np.array(sc.pbc, np.int32)
    src = np.ascontiguousarray(sc.bond_src, np.int32)
    dst = np.ascontiguousarray(sc.bond_dst, np.int32)
    R = np.ascontiguousarray(sc.bond_R, np.int32).reshape(-1)
    typ_of = np.arange(len(src), dtype=np.int32)
    ptr = np.zeros(sc.N + 1, np.int64)
    nnz = lib.oracle_stencil_csr(sc.ns, _p(L, ip), _p(pbc, ip), len(src), _p(src, ip), _p(dst, ip), _p(R, ip),
                                 _p(typ_of, ip), _p(ptr, C.POINTER(C.c_int64)), None, None)
    nbr = np.zeros(nnz, np.int32)
    typ = np.zeros(nnz, np.int32)
    lib.oracle_stencil_csr(sc.ns, _p(L, ip), _p(pbc, ip), len(src), _p(src, ip), _p(dst, ip), _p(R, ip),
                           _p(typ_of, ip), _p(ptr, C.POINTER(C.c_int64)), _p(nbr, ip), _p(typ, ip))
    return ptr, nbr, typ, np.ascontiguousarray(sc.table, np.float64), sc.width


class OracleLLG:
    """CPU restatement of magex LLGSolver (heun / depondt) on a Supercell.

    csr="blocks" uses Supercell.neighbour_csr() (magex's sorted, merged block list: closest to the
    reference summation order); csr="stencil" uses the C builder (for large supercells).
    """

    def __init__(self, sc, alpha=0.1, dt=1e-3, temperature=0.0, seed=None, precession=True,
                 integrator="heun", noise="host", threads=0, csr="blocks", tuned=False):
        self.lib = load(tuned)
        self.sc = sc
        N = sc.N
        if csr == "blocks":
            ptr, nbr, typ, table = sc.neighbour_csr()
            width = 9
        else:
            ptr, nbr, typ, table, width = stencil_csr(sc)
        self._arrays = dict(ptr=np.ascontiguousarray(ptr, np.int64), nbr=np.ascontiguousarray(nbr, np.int32),
                            typ=np.ascontiguousarray(typ, np.int32), table=np.ascontiguousarray(table, np.float64))
        A = sc.A if sc.has_A else None
        self._arrays["A"] = None if A is None else np.ascontiguousarray(A, np.float64).reshape(-1)
        self._arrays["mu"] = np.ascontiguousarray(sc.mu, np.float64)
        pin = None if sc.pinned is None else np.ascontiguousarray(np.asarray(sc.pinned, bool), np.uint8)
        self._arrays["pinned"] = pin
        m = _Model()
        m.N = N
        m.ptr = _p(self._arrays["ptr"], C.POINTER(C.c_int64))
        m.nbr = _p(self._arrays["nbr"], C.POINTER(C.c_int32))
        m.typ = _p(self._arrays["typ"], C.POINTER(C.c_int32))
        m.table = _p(self._arrays["table"])
        m.width = width
        m.A = _p(self._arrays["A"])
        m.mu = _p(self._arrays["mu"])
        m.B[:] = [float(x) for x in sc.B]
        m.pinned = _p(pin, C.POINTER(C.c_uint8))
        cub, uni = getattr(sc, "cubic", None), getattr(sc, "uniaxial_higher", None)
        if cub is not None:
            self._arrays["Kc"] = np.ascontiguousarray(np.broadcast_to(np.asarray(cub[0], float), (N,)))
            m.Kc = _p(self._arrays["Kc"])
            m.C[:] = [float(x) for x in np.asarray(cub[1], float).reshape(9)]
        if uni is not None:
            self._arrays["K2"] = np.ascontiguousarray(np.broadcast_to(np.asarray(uni[0], float), (N,)))
            self._arrays["K3"] = np.ascontiguousarray(np.broadcast_to(np.asarray(uni[1], float), (N,)))
            m.K2, m.K3 = _p(self._arrays["K2"]), _p(self._arrays["K3"])
            m.u[:] = [float(x) for x in np.asarray(uni[2], float).reshape(3)]
        self._m = m
        a = getattr(sc, "alpha_site", None)
        al = np.asarray(a if (a is not None and np.isscalar(alpha)) else alpha, float)
        if al.ndim and a is not None and np.isscalar(alpha):
            al = np.where(np.isnan(al), float(alpha), al)
        self.alpha = al
        self._alpha_arr = np.ascontiguousarray(np.broadcast_to(al, (N,)), np.float64)
        self.dt = float(dt)
        self.T = float(temperature)
        self.rng = np.random.default_rng(seed)
        self.precession = bool(precession)
        self.depondt = integrator == "depondt"
        if integrator not in ("heun", "depondt"):
            raise ValueError("oracle implements heun and depondt")
        self.noise = noise
        self.threads = int(threads)
        self.time = 0.0
        self._ep = np.empty((N, 3))
        self._k1 = np.empty((N, 3))
        self._b = np.empty((N, 3))
        if noise == "ziggurat":
            ss = np.random.SeedSequence(int(seed) if seed is not None else None)
            st = ss.generate_state(256, dtype=np.uint64)
            st[st == 0] = np.uint64(0x9E3779B97F4A7C15)
            self._streams = np.ascontiguousarray(st)

    def sigma(self):
        sc = self.sc
        sT = getattr(sc, "site_T", None)
        T = self.T if sT is None else np.where(np.isnan(sT), self.T, sT)
        return np.sqrt(2.0 * self.alpha * K_B * T / (GAMMA * sc.mu * MU_B * self.dt))

    def noisy(self):
        return self.T > 0 or getattr(self.sc, "site_T", None) is not None

    def thermal_field(self):
        """(N,3) b in tesla, or None at T = 0 (no draw), as magex/llg.py:106-122."""
        if not self.noisy():
            return None
        sig = np.ascontiguousarray(np.broadcast_to(self.sigma(), (self.sc.N,)), np.float64)
        if self.noise == "host":
            b = sig[:, None] * self.rng.normal(size=(self.sc.N, 3))
            if self.sc.pinned is not None:
                b[np.asarray(self.sc.pinned, bool)] = 0.0
            return np.ascontiguousarray(b)
        pin = self._arrays["pinned"]
        self.lib.oracle_gauss3(_p(self._b), self._streams.ctypes.data_as(C.POINTER(C.c_uint64)), 256, _p(sig),
                               _p(pin, C.POINTER(C.c_uint8)), self.sc.N, self.threads)
        return self._b

    def step(self, e):
        """One step; returns a new (N,3) array (the input is left unchanged)."""
        out = np.array(e, dtype=np.float64, order="C", copy=True)
        self.step_inplace(out)
        return out

    def step_inplace(self, e, b="draw"):
        self._m.B[:] = [float(x) for x in self.sc.B]
        if isinstance(b, str):
            b = self.thermal_field()
        self.lib.oracle_step(C.byref(self._m), _p(self._alpha_arr), self.dt, int(self.precession), int(self.depondt),
                             _p(b), _p(e), _p(self._ep), _p(self._k1), self.threads)
        self.time += self.dt
        return e

    def stage(self, e, b, stage):
        """Predictor (stage 0: e -> self.ep, self.k1) or corrector (stage 1: e updated in place from
        self.ep, self.k1) with the given thermal field b ((N, 3) or None)."""
        self._m.B[:] = [float(x) for x in self.sc.B]
        self.lib.oracle_stage(C.byref(self._m), _p(self._alpha_arr), self.dt, int(self.precession), int(self.depondt),
                              _p(b), _p(e), _p(self._ep), _p(self._k1), int(stage), self.threads)
        return e

    @property
    def ep(self):
        return self._ep

    def observables(self, e):
        e = np.ascontiguousarray(e, np.float64)
        out = np.zeros(8)
        sg = np.ascontiguousarray(self.sc.signs, np.float64)
        self._m.B[:] = [float(x) for x in self.sc.B]
        self.lib.oracle_observables(C.byref(self._m), _p(e), _p(sg), _p(out), self.threads)
        return out

    def row(self, e):
        o = self.observables(e)
        N = self.sc.N
        return [self.time, o[0] / N, o[1] / N, o[2] / N, o[3] / N, float(np.linalg.norm(o[4:7]) / N), float(o[7])]


class OracleMC:
    """CPU restatement of magex's MetropolisMC NumPy sweep (magex/montecarlo.py:71-230): greedy colour
    classes, trial moves gaussian / uniform / heatbath / hinzke, over-relaxation passes, with the draws
    made by ``numpy.random.default_rng(seed)`` in magex's order (so it reproduces magex's trajectory).
    Built on OracleLLG's model arrays (same neighbour lists)."""

    MOVES = {"gaussian": 0, "uniform": 1, "heatbath": 2, "hinzke": 3}

    def __init__(self, sc, temperature, seed=None, sigma=0.6, overrelax=1, move="gaussian", threads=0,
                 csr="blocks"):
        self.llg = OracleLLG(sc, csr=csr, threads=threads)
        self.lib = self.llg.lib
        self.sc = sc
        a = self.llg._arrays
        col = np.empty(sc.N, np.int32)
        ip = C.POINTER(C.c_int32)
        nc = self.lib.oracle_greedy_colour(sc.N, _p(a["ptr"], C.POINTER(C.c_int64)), _p(a["nbr"], ip), _p(col, ip))
        self.colour = col
        pinned = None if getattr(sc, "pinned", None) is None else np.asarray(sc.pinned, bool)
        self.groups = []
        for c in range(nc):
            idx = np.flatnonzero(col == c).astype(np.int64)
            if pinned is not None:
                idx = idx[~pinned[idx]]
            if len(idx):
                self.groups.append(np.ascontiguousarray(idx))
        self.ncolors = len(self.groups)
        self.T = float(temperature)
        self.rng = np.random.default_rng(seed)
        self.sigma = float(sigma)
        self.overrelax = int(overrelax)
        self.move = move
        self.threads = int(threads)
        self.accepted = 0
        self.tried = 0

    def _beta(self):
        sT = getattr(self.sc, "site_T", None)
        if sT is not None:
            T = np.where(np.isnan(sT), self.T, sT)
            return np.ascontiguousarray(1.0 / (K_B * np.maximum(T, 1e-9)))
        b = 1.0 / (K_B * self.T) if self.T > 0 else np.inf
        return np.full(self.sc.N, b)

    def _group(self, e, idx, mv, draws, beta):
        return int(self.lib.oracle_mc_group(C.byref(self.llg._m), _p(idx, C.POINTER(C.c_int64)), len(idx), mv,
                                            _p(beta), self.sigma, _p(np.ascontiguousarray(draws, np.float64)),
                                            _p(e), self.threads))

    def sweep(self, e):
        """One sweep of e ((N, 3) float64 C-contiguous array), in place."""
        rng = self.rng
        beta = self._beta()
        self.llg._m.B[:] = [float(x) for x in self.sc.B]
        for idx in self.groups:
            n = len(idx)
            if self.move == "heatbath" and np.all(np.isfinite(beta[idx])):
                mv, parts = 2, [rng.random(n), rng.random(n)]
            elif self.move == "hinzke":
                mv, parts = 3, [rng.integers(0, 3, n).astype(np.float64), rng.normal(size=(n, 3)).ravel(),
                                rng.normal(size=(n, 3)).ravel()]
            else:
                mv, parts = (1 if self.move == "uniform" else 0), [rng.normal(size=(n, 3)).ravel()]
            parts.append(rng.random(n))
            self.accepted += self._group(e, idx, mv, np.concatenate(parts), beta)
            self.tried += n
        for _ in range(self.overrelax):
            for idx in self.groups:
                self._group(e, idx, 4, rng.random(len(idx)), beta)
        return e


def solid_angle_charge(e, tri, sign):
    """Skyrmion number (1/4 pi) sum_t sign_t * 2 atan2(s1.(s2 x s3), 1 + s1.s2 + s2.s3 + s3.s1) over
    triangles tri ((T, 3) site indices of spins e, (N, 3)), the Berg-Luscher solid angle of
    magex/texture.py:53-62 with the plane's handedness folded into sign."""
    e = np.asarray(e, np.float64)
    tri = np.asarray(tri, np.int64).reshape(-1, 3)
    s1, s2, s3 = e[tri[:, 0]], e[tri[:, 1]], e[tri[:, 2]]
    num = np.einsum("ij,ij->i", s1, np.cross(s2, s3))
    den = 1 + np.einsum("ij,ij->i", s1, s2) + np.einsum("ij,ij->i", s2, s3) + np.einsum("ij,ij->i", s3, s1)
    return float((2 * np.arctan2(num, den) * np.asarray(sign, np.float64)).sum() / (4 * np.pi))
