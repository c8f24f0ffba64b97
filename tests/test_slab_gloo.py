"""Slab decomposition of one lattice with halo exchanges (magex/mpi_spin.py:150-180) on CPU: two and
three gloo ranks step their slabs with the oracle's predictor / corrector, exchange the halo layers
of ep and e through magex_gb300.slab.DistTransport, and must reproduce the unsplit oracle run (same
noise draws) to rounding, with the whole-lattice observables from the reduced partials."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


CASES = {
    # name: (model key, L, pbc, field, alpha, dt, T, steps)
    "bcc_periodic": ("bcc2", (6, 3, 3), (1, 1, 1), (0.0, 0.0, 0.5), 0.05, 1e-4, 300.0, 6),
    "sc_open": ("sc_open", (7, 3, 2), (0, 0, 0), (0.2, 0.0, 2.0), 0.1, 1e-3, 10.0, 6),
    "tri_two_shell": ("tri_two_shell", (9, 4, 1), (1, 1, 0), (0.0, 0.0, 1.0), 0.2, 1e-3, 5.0, 5),
}


class OracleSlab:
    """The oracle as a slab engine: local supercell (owned + halo layers), magex-order arrays."""

    def __init__(self, uc, L, pbc, field, alpha, dt, rank, world):
        from magex_gb300.lattice import Supercell
        from magex_gb300.slab import SlabGeometry, halo_depth
        from oracle import OracleLLG
        self.geo = SlabGeometry(L, pbc, halo_depth(Supercell(uc, L, pbc, field)), world, rank)
        self.sc = Supercell(uc, self.geo.L_local, self.geo.pbc_local, field)
        self.ora = OracleLLG(self.sc, alpha, dt, 0.0, None, csr="stencil")
        self.sites = self.geo.global_sites(self.sc.ns)
        self.layer = self.sc.L[1] * self.sc.L[2] * self.sc.ns

    def _arr(self, which, e):
        return self.ora.ep if which == "ep" else e

    def pack(self, which, e):
        g, x, out = self.geo, self._arr(which, e), {}
        a, b = g.own
        if g.left_rank is not None:
            out["left"] = torch.as_tensor(x[a * self.layer:(a + g.h) * self.layer].copy())
        if g.right_rank is not None:
            out["right"] = torch.as_tensor(x[(b - g.h) * self.layer:b * self.layer].copy())
        return out

    def unpack(self, which, e, recv):
        g, x = self.geo, self._arr(which, e)
        if "left" in recv:
            x[:g.hl * self.layer] = recv["left"].numpy()
        if "right" in recv:
            x[g.own[1] * self.layer:(g.own[1] + g.hr) * self.layer] = recv["right"].numpy()


def _worker(rank, world, port, case, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    for p in (root, os.path.join(root, "oracle"), os.path.join(root, "tests")):
        sys.path.insert(0, p)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from magex_gb300.slab import DistTransport
        e_all, sigma, uc, (key, L, pbc, B, alpha, dt, T, steps) = case
        sl = OracleSlab(uc, L, pbc, B, alpha, dt, rank, world)
        tr = DistTransport()
        e = np.ascontiguousarray(e_all[sl.sites])
        rng = np.random.default_rng(11)
        for _ in range(steps):
            b = np.ascontiguousarray((sigma[:, None] * rng.normal(size=e_all.shape))[sl.sites])
            sl.ora.stage(e, b, 0)
            (r,) = tr.exchange([sl], [sl.pack("ep", e)])
            sl.unpack("ep", e, r)
            sl.ora.stage(e, b, 1)
            (r,) = tr.exchange([sl], [sl.pack("e", e)])
            sl.unpack("e", e, r)
        owned = e[sl.geo.owned_rows(sl.sc.ns)]
        # partial observables reduce to sums (E, spin sums) and a max (torque) over the ranks
        red = tr.reduce([np.arange(8, dtype=np.float64) * (rank + 1)])
        q.put((rank, sl.geo.start, owned, red))
    finally:
        dist.destroy_process_group()


def _reference(case):
    from oracle import OracleLLG
    from magex_gb300.lattice import Supercell
    e_all, sigma, uc, (key, L, pbc, B, alpha, dt, T, steps) = case
    sc = Supercell(uc, L, pbc, B)
    ora = OracleLLG(sc, alpha, dt, 0.0, None, csr="stencil")
    e = e_all.copy()
    rng = np.random.default_rng(11)
    for _ in range(steps):
        b = np.ascontiguousarray(sigma[:, None] * rng.normal(size=e_all.shape))
        ora.step_inplace(e, b)
    return e, ora.observables(e)


@pytest.mark.parametrize("name,world", [("bcc_periodic", 2), ("bcc_periodic", 3), ("sc_open", 2),
                                        ("sc_open", 3), ("tri_two_shell", 2)])
def test_slab_decomposition_matches_unsplit_oracle(golden_models, name, world):
    from magex_gb300.constants import GAMMA, K_B, MU_B
    from magex_gb300.lattice import Supercell
    from magex_gb300.spinmodel import load_results
    spec = CASES[name]
    key, L, pbc, B, alpha, dt, T, steps = spec
    uc = load_results(golden_models[key]["model"])
    sc = Supercell(uc, L, pbc, B)
    e_all = sc.init_spins("random", seed=4)
    sigma = np.sqrt(2 * alpha * K_B * T / (GAMMA * np.asarray(sc.mu) * MU_B * dt))
    case = (e_all, sigma, uc, spec)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, case, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted([q.get(timeout=180) for _ in range(world)], key=lambda r: r[0])
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    ref, _ = _reference(case)
    split = np.concatenate([r[2] for r in res])
    assert split.shape == ref.shape
    assert np.abs(split - ref).max() <= 1e-15 * steps
    tot = sum(range(1, world + 1))
    for r in res:
        np.testing.assert_array_equal(r[3][:7], np.arange(7) * tot)
        assert r[3][7] == 7 * world


def _silent_peer_worker(rank, world, port, spec_uc, q, done):
    """Rank 1 joins the group but never sends its halo; rank 0 must get an error, not wait forever."""
    import datetime
    import time
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    for p in (root, os.path.join(root, "oracle"), os.path.join(root, "tests")):
        sys.path.insert(0, p)
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=datetime.timedelta(seconds=3))
    if rank == 1:
        done.wait(120)          # stay connected until rank 0 has given up, then leave
        return
    from magex_gb300.slab import DistTransport
    uc, (key, L, pbc, B, alpha, dt, T, steps) = spec_uc
    sl = OracleSlab(uc, L, pbc, B, alpha, dt, rank, world)
    e = np.zeros((sl.sc.N, 3))
    e[:, 2] = 1.0
    t0 = time.time()
    try:
        DistTransport().exchange([sl], [sl.pack("e", e)])
        q.put(("returned", time.time() - t0, ""))
    except Exception as err:                      # the process group's timeout ends the receive
        q.put(("error", time.time() - t0, type(err).__name__))
    finally:
        done.set()


def test_missing_halo_message_raises_instead_of_hanging(golden_models):
    """Failure detection on the host: a neighbour that never sends its halo layers makes the
    exchange raise once the process group's timeout (3 s here) expires; magex's MPI exchange would
    block forever in Waitall (magex/mpi_spin.py:102)."""
    from magex_gb300.spinmodel import load_results
    spec = CASES["bcc_periodic"]
    uc = load_results(golden_models[spec[0]]["model"])
    ctx = mp.get_context("spawn")
    q, done = ctx.Queue(), ctx.Event()
    port = _free_port()
    procs = [ctx.Process(target=_silent_peer_worker, args=(r, 2, port, (uc, spec), q, done)) for r in range(2)]
    for p in procs:
        p.start()
    status, elapsed, what = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        if p.is_alive():
            p.kill()
    assert status == "error", (status, elapsed, what)
    assert elapsed < 60
