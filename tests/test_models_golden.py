"""Host model layer against the reference: make_model dicts, load_results couplings, supercell folding."""
import numpy as np
import pytest

from magex_gb300.lattice import Supercell, compress_tensors
from magex_gb300.spinmodel import load_results, make_model

MODEL_NAMES = ["sc", "sc_dmi", "sc_two_shell", "sc_afm", "sc_open", "tri", "tri_two_shell", "honeycomb_bulk",
               "bcc1", "fcc_jani", "kagome"]


@pytest.mark.parametrize("name", MODEL_NAMES)
def test_make_model_matches_reference(golden_models, name):
    kw = golden_models[name + "__kwargs"]
    mine = make_model(**kw)
    ref = golden_models[name]["model"]
    assert mine.keys() == ref.keys()
    for k in ref:
        if k == "pairs":
            assert len(mine[k]) == len(ref[k])
            for a, b in zip(mine[k], ref[k]):
                assert a == b
        else:
            assert np.array_equal(np.asarray(mine[k], dtype=object), np.asarray(ref[k], dtype=object)) or mine[k] == ref[k], k


@pytest.mark.parametrize("name", MODEL_NAMES + ["bcc2", "bcc2_shell4", "free"])
def test_load_results_matches_reference(golden_models, name):
    ref = golden_models[name]
    uc = load_results(ref["model"])
    assert len(uc.couplings) == len(ref["couplings"])
    for (i, j, R, J), (ri, rj, rR, rJ) in zip(uc.couplings, ref["couplings"]):
        assert (i, j) == (ri, rj)
        assert list(R) == rR
        assert np.array_equal(J, np.array(rJ))
    assert np.array_equal(uc.A, np.array(ref["A"]))
    assert np.array_equal(uc.moments, np.array(ref["moments"]))
    assert np.array_equal(uc.signs, np.array(ref["signs"]))
    for k, v in ref["info"].items():
        assert uc.info[k] == v, k


def test_bcc_two_site_shells(golden_models):
    uc = load_results(golden_models["bcc2"]["model"])
    assert uc.info["ncouplings_per_cell"] == 52              # 2 sites x (8 + 6 + 12)
    uc4 = load_results(golden_models["bcc2_shell4"]["model"])
    assert uc4.info["ncouplings_per_cell"] == 100            # 2 sites x (8 + 6 + 12 + 24)
    # reverse bonds carry the transpose (exact gradient)
    J = {(i, j, tuple(R)): T for i, j, R, T in uc.couplings}
    for (i, j, R), T in J.items():
        assert np.array_equal(J[(j, i, tuple(-x for x in R))], T.T)


def test_compress_tensors_exact():
    iso = [np.eye(3) * 2.0, np.eye(3) * -1.0]
    w, t = compress_tensors(iso)
    assert w == 1 and np.array_equal(t[:, 0], [2.0, -1.0])
    from magex_gb300.spinmodel import skew
    dmi = [np.eye(3) + skew([0.1, -0.2, 0.3])]
    w, t = compress_tensors(dmi)
    assert w == 4 and np.array_equal(t[0], [1.0, 0.1, -0.2, 0.3])
    full = [np.eye(3) + np.diag([0.0, 1e-3, 0.0])]
    w, t = compress_tensors(full)
    assert w == 9


def test_self_image_folding_and_open_bounds(golden_models):
    uc = load_results(golden_models["sc_two_shell"]["model"])
    sc = Supercell(uc, (1, 2, 3), (True, True, True))
    # the +-x nearest neighbours and the (+-1, 0, 0)-containing second-shell bonds with R0 % 1 == 0 and
    # R1 % 2 == 0, R2 % 3 == 0 reach their own image: (+-1,0,0) only
    assert sc.self_folded == 2 * sc.ncell
    Jx = [J for i, j, R, J in uc.couplings if list(R) in ([1, 0, 0], [-1, 0, 0])]
    A = np.array(uc.A[0]).copy()
    for J in Jx:
        A -= 0.5 * (J + J.T)
    assert np.allclose(sc.A_sub[0], A, rtol=0, atol=1e-15)
    ucq = load_results(golden_models["sc_open"]["model"])
    sco = Supercell(ucq, (5, 5, 4), (False, False, False))
    ptr, nbr, typ, table = sco.neighbour_csr()
    deg = np.diff(ptr)
    assert deg.min() == 3 and deg.max() == 6                 # corners 3, bulk 6


def test_init_spins_matches_reference(golden, golden_models):
    from helpers import golden_supercell
    for tag in ("sc16", "bcc2_thermal", "tri16", "sc_structure"):
        sc, meta = golden_supercell(golden_models, tag)
        e0 = sc.init_spins("random", seed=meta["init_seed"])
        assert np.array_equal(e0, golden[f"{tag}/e0"]), tag


def test_onsite_terms_of_a_magex_system_are_carried(golden_models):
    """The first cubic and the first higher-uniaxial term of a magex system go to the kernels (as
    magex/fast.py:647-652 splits them off); other terms are refused."""
    import numpy as np
    import pytest
    from magex_gb300.device import _take_onsite_terms
    from magex_gb300.lattice import Supercell
    from magex_gb300.spinmodel import load_results

    class CubicAnisotropy:
        def __init__(self, Kc, C):
            self.Kc, self.C = Kc, C

    class UniaxialHigher:
        def __init__(self, K2, K3, u):
            self.K2, self.K3, self.u = K2, K3, u

    class Dipolar:
        pass

    sc = Supercell(load_results(golden_models["sc"]["model"]), (2, 2, 2))
    Kc = np.linspace(0.1, 0.8, sc.N)
    _take_onsite_terms(sc, [CubicAnisotropy(Kc, np.eye(3)), UniaxialHigher(np.ones(sc.N), np.zeros(sc.N), [0, 0, 1.0])])
    assert np.array_equal(sc.cubic[0], Kc) and np.array_equal(sc.cubic[1], np.eye(3))
    assert np.array_equal(sc.uniaxial_higher[2], [0, 0, 1.0]) and sc.terms == []
    sc2 = Supercell(load_results(golden_models["sc"]["model"]), (2, 2, 2))
    with pytest.raises(NotImplementedError):
        _take_onsite_terms(sc2, [Dipolar()])
