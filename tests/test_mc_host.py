"""Monte Carlo host logic (CPU): the native greedy colouring against magex's own colour classes and
the T_c estimator against magex's estimate_tc, on the reference's recorded outputs."""
import numpy as np
import pytest

from helpers import MC_TAGS as TAGS, mc_system


@pytest.mark.parametrize("tag", TAGS)
def test_colouring_matches_reference(golden, golden_models, tag):
    from magex_gb300.mc import colouring
    sc, meta = mc_system(golden, golden_models, tag)
    col, nc = colouring(sc)
    ref = golden[f"mc/{tag}/colour"]
    assert col.shape == ref.shape and np.array_equal(col, ref)
    assert nc == int(ref.max()) + 1


def test_colouring_is_proper_on_a_large_bcc_lattice():
    """No coupling joins two sites of one colour (every class can be updated at once)."""
    from magex_gb300.mc import colouring
    from magex_gb300.workloads import bcc_two_site
    sc = bcc_two_site(L=12)
    col, nc = colouring(sc)
    ptr, nbr, _, _ = sc.neighbour_csr()
    rows = np.repeat(np.arange(sc.N), np.diff(ptr))
    other = rows != nbr
    assert not np.any(col[rows[other]] == col[nbr[other]])
    assert 2 <= nc <= 32


def test_estimate_tc_matches_reference(golden_models):
    from magex_gb300.mc import estimate_tc
    g = golden_models["mc_tc"]
    est = estimate_tc(g["rows"])
    ref = g["estimate"]
    assert est["method"] == ref["method"]
    assert abs(est["Tc"] - ref["Tc"]) < 1e-12
    for k in ("chi_peak", "C_peak"):
        for L, v in ref[k].items():
            assert abs(est[k][L] - v) < 1e-12, (k, L)
    assert len(est["binder"]) == len(ref["binder"])
    for mine, theirs in zip(est["binder"], ref["binder"]):
        assert mine["sizes"] == theirs["sizes"]
        assert mine["T"] == pytest.approx(theirs["T"], abs=1e-12)


def test_mc_entry_points_exported():
    from magex_gb300 import _lib
    lib = _lib.load()
    for name in ("mgx_colour_stencil", "mgx_colour_graph", "mgx_mc_create", "mgx_mc_destroy", "mgx_mc_set_beta",
                 "mgx_mc_set_sigma", "mgx_mc_host_draws", "mgx_mc_sweep", "mgx_mc_counts"):
        assert hasattr(lib, name)
