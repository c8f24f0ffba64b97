"""Output writers (CPU): files byte-for-byte equal to those magex's own writers produced for the same
system and spins (SHA-256 recorded by tests/golden/make_golden.py), and a large-N round trip."""
import hashlib

import numpy as np
import pytest


def _digest(path):
    with open(path, "rb") as f:
        data = f.read()
    return dict(sha256=hashlib.sha256(data).hexdigest(), size=len(data))


@pytest.mark.parametrize("tag", ["tri", "bcc2"])
def test_writers_match_reference_bytes(golden, golden_models, tmp_path, tag):
    from magex_gb300.lattice import Supercell
    from magex_gb300.output import save_spins, write_ovf_atomistic, write_vtk, write_xyz
    from magex_gb300.spinmodel import load_results
    meta = golden_models["outputs"][tag]
    sc = Supercell(load_results(golden_models[tag]["model"]), tuple(meta["L"]), tuple(meta["pbc"]), (0.0, 0.0, 0.5))
    e = golden[f"out/{tag}/e"]
    p = str(tmp_path / tag)
    write_xyz(p + ".xyz", sc, e, comment="t=1.5 ps")
    write_vtk(p + ".vtk", sc, e, extra=dict(E=np.linspace(-3, 4e-6, sc.N)))
    write_ovf_atomistic(p + ".ovf", sc, e)
    save_spins(p + ".npz", sc, e)
    for name in ("xyz", "vtk", "ovf", "csv"):
        assert _digest(f"{p}.{name}") == meta["files"][name], name
    z = np.load(p + ".npz")
    assert np.array_equal(z["spins"], e) and np.array_equal(z["positions"], sc.positions)
    assert np.array_equal(z["supercell"], np.array(sc.L))


def test_table_matches_reference_bytes(golden, golden_models, tmp_path):
    from magex_gb300.output import write_table
    p = str(tmp_path / "table.csv")
    write_table(p, golden["sc16/table"])
    assert _digest(p) == golden_models["outputs"]["table"]


def test_large_write_round_trip(tmp_path):
    """1,048,576 spins (16 formatting chunks): the CSV reads back to 6 decimals, the xyz has N + 2 lines."""
    from magex_gb300.output import save_spins, write_xyz
    from magex_gb300.workloads import bcc_two_site
    sc = bcc_two_site(L=64)
    e = sc.init_spins("random", seed=3)
    p = str(tmp_path / "big.npz")
    save_spins(p, sc, e)
    back = np.loadtxt(p.replace(".npz", ".csv"), delimiter=",", skiprows=1)
    assert back.shape == (sc.N, 6)
    assert np.abs(back[:, 3:] - e).max() <= 5e-7 + 1e-12
    assert np.abs(back[:, :3] - sc.positions).max() <= 5e-7 + 1e-9
    q = str(tmp_path / "big.xyz")
    write_xyz(q, sc, e)
    with open(q) as f:
        assert sum(1 for _ in f) == sc.N + 2


def test_writer_errors():
    from magex_gb300 import _lib
    lib = _lib.load()
    assert lib.mgx_write_csv(b"/nonexistent-dir/x.csv", 1, 1, _lib.dptr(np.zeros(1)), b"%.6f", None) == _lib.MGX_ERR_INVALID
    assert lib.mgx_write_csv(b"x.csv", 1, 1, _lib.dptr(np.zeros(1)), b"%s", None) == _lib.MGX_ERR_INVALID
