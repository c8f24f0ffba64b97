"""Topological charge of one layer: magex_gb300.texture against magex/texture.py:14-63.

The triangulation (periodic Delaunay, centroid rule, orientation and handedness signs) is host code;
it is checked here on the CPU against the reference's charges through the oracle's solid-angle sum.
The device sum over the same triangles is checked in the GPU test."""
import numpy as np
import pytest
import scipy

from magex_gb300.lattice import Supercell
from magex_gb300.spinmodel import load_results
from magex_gb300 import texture

CASES = ("square", "honeycomb", "kagome", "sc_xz", "sc_open")


def _system(golden_models, tag):
    c = golden_models["topo2"][tag]
    sc = Supercell(load_results(golden_models[c["model"]]["model"]), tuple(c["L"]), tuple(c["pbc"]))
    return sc, c["plane"], c["layer"]


def _same_qhull(golden):
    return str(golden["scipy_version"]) == scipy.__version__


@pytest.mark.parametrize("tag", CASES)
def test_layer_triangles_match_reference(golden, golden_models, tag):
    from oracle import solid_angle_charge
    if not _same_qhull(golden):
        pytest.skip("charges were written with another scipy (qhull) version")
    sc, plane, layer = _system(golden_models, tag)
    tri, sign = texture.layer_triangles(sc, plane, layer)
    assert tri.min() >= 0 and tri.max() < sc.N
    for k in ("bubble", "random"):
        Q = solid_angle_charge(golden[f"topo2/{tag}/{k}_e"], tri, sign)
        assert abs(Q - float(golden[f"topo2/{tag}/{k}_Q"])) < 1e-12, (tag, k)


def test_layer_indices(golden_models):
    sc = Supercell(load_results(golden_models["sc"]["model"]), (2, 3, 4), (True, True, False))
    z = sc.positions[:, 2]
    for layer, level in ((0, z.min()), (-1, z.max()), (2, np.unique(z)[2])):
        idx, axes, nlev = texture.layer_indices(sc, "xy", layer)
        assert nlev == 4 and axes == (0, 1, 2) and len(idx) == 6
        assert np.all(z[idx] == level)


def test_too_few_spins_is_zero(golden_models):
    sc = Supercell(load_results(golden_models["sc"]["model"]), (1, 1, 4), (True, True, True))
    assert texture.layer_triangles(sc, "xy", 0) is None
    assert texture.topological_charge(sc, np.tile([0.0, 0.0, 1.0], (sc.N, 1)), "xy", 0) == 0.0


@pytest.mark.gpu
@pytest.mark.parametrize("tag", CASES)
def test_device_charge(cuda, golden, golden_models, tag):
    import torch
    from oracle import solid_angle_charge
    sc, plane, layer = _system(golden_models, tag)
    tri, sign = texture.layer_triangles(sc, plane, layer)
    for k in ("bubble", "random"):
        e = golden[f"topo2/{tag}/{k}_e"]
        Q = texture.topological_charge(sc, e, plane, layer)
        assert abs(Q - solid_angle_charge(e, tri, sign)) < 1e-12, (tag, k)
        if _same_qhull(golden):
            assert abs(Q - float(golden[f"topo2/{tag}/{k}_Q"])) < 1e-9, (tag, k)
        # a device tensor, and the kept triangulation on the second call
        assert texture.topological_charge(sc, torch.as_tensor(e, device="cuda"), plane, layer) == Q


TEXTURES = ("skyrmion", "skyrmions", "helicity0", "antiskyrmion")


def _film40(golden_models):
    return Supercell(load_results(golden_models["tri"]["model"]), (40, 40, 1), (True, True, False), (0, 0, 1.0))


def test_texture_charges_match_reference(golden, golden_models):
    from oracle import solid_angle_charge
    sc = _film40(golden_models)
    tri, sign = texture.layer_triangles(sc)
    for k in TEXTURES:
        Q = solid_angle_charge(golden[f"topo3/{k}_e"], tri, sign)
        assert abs(Q - float(golden[f"topo3/{k}_Q"])) < 1e-12, k


@pytest.mark.gpu
def test_texture_charges_on_device(cuda, golden, golden_models):
    """The assertions of tests/test_universal.py:81-91 on magex's own textures, through the drop-in."""
    sc = _film40(golden_models)
    Q = {k: texture.topological_charge(sc, golden[f"topo3/{k}_e"], "xy", 0) for k in TEXTURES}
    for k in TEXTURES:
        assert abs(Q[k] - float(golden[f"topo3/{k}_Q"])) < 1e-9, k
    assert abs(abs(Q["skyrmion"]) - 1) < 1e-6
    assert abs(abs(Q["skyrmions"]) - 2) < 1e-6
    assert abs(Q["helicity0"] + Q["antiskyrmion"]) < 1e-6
    assert abs(texture.topological_charge(sc, np.tile([0, 0, 1.0], (sc.N, 1)))) < 1e-9
