"""Arbitrary lattices (per-site neighbour lists): host construction and the oracle against the reference."""
import numpy as np
import pytest

from helpers import golden_irregular
from oracle import OracleLLG


@pytest.mark.parametrize("tag", ["sc_sphere", "sc_interface"])
def test_neighbour_list_reproduces_matrix(golden, golden_models, tag):
    nl, meta, J = golden_irregular(golden, golden_models, tag)
    ptr, nbr, typ, table = nl.neighbour_csr()
    rows = np.repeat(np.arange(nl.N), np.diff(ptr))
    dense = np.zeros((3 * nl.N, 3 * nl.N))
    blocks = table[typ].reshape(-1, 3, 3)
    for r, c, B in zip(rows, nbr, blocks):
        dense[3 * r:3 * r + 3, 3 * c:3 * c + 3] += B
    assert np.array_equal(dense, J.toarray())


@pytest.mark.parametrize("tag", ["sc_sphere", "sc_interface"])
def test_oracle_on_irregular_lattice(golden, golden_models, tag):
    nl, meta, _ = golden_irregular(golden, golden_models, tag)
    ora = OracleLLG(nl, meta["alpha"], meta["dt"], meta["T"], meta["seed"])
    e = golden[f"{tag}/e0"].copy()
    for _ in range(meta["steps"]):
        e = ora.step(e)
    assert np.abs(e - golden[f"{tag}/e{meta['steps']}"]).max() <= 1e-12 * meta["steps"]
    E = float(golden[f"{tag}/energy"])
    assert abs(ora.observables(e)[0] - E) <= 1e-12 * abs(E)


def test_spin_system_routes_to_neighbour_list(golden, golden_models):
    """A SpinSystem whose matrix is not its unit cell's stencil (carved) becomes a NeighbourList."""
    from types import SimpleNamespace

    from magex_gb300.device import supercell_from_system
    from magex_gb300.lattice import NeighbourList
    from magex_gb300.spinmodel import load_results
    nl, meta, J = golden_irregular(golden, golden_models, "sc_sphere")
    uc = load_results(golden_models["sc_dmi"]["model"])
    fake = SimpleNamespace(uc=uc, L=tuple(meta["L"]), pbc=tuple(meta["pbc"]), N=nl.N, Jsp=J, B=np.array(meta["B"]),
                           mu=golden["sc_sphere/mu"], A=golden["sc_sphere/A"], signs=golden["sc_sphere/signs"],
                           pinned=None, site_T=None, alpha_site=None, terms=[], has_higher=False)
    sc = supercell_from_system(fake)
    assert isinstance(sc, NeighbourList) and sc.N == nl.N
