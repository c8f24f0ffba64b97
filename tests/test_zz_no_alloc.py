"""mgx_llg_step_noalloc: the Heun step for callers that cannot allocate GPU memory.

Such callers (a framework that owns all device memory through its own pool and hands a plugin only
its input and output buffers, a real-time loop that must not wait on the allocator) get a step whose
scratch lives in a fixed static device array.  These tests call it through the C ABI and compare it
with the planned entry point (mgx_llg_create + mgx_llg_step, via GB300LLG) on the same spins and the
same noise, and with the reference's own trajectories (golden fixtures made by running magex), for
two or more calls in a row, to the 1e-12 per-step tolerance of the other GPU tests.  The file is named
so that pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

ALPHA, DT, TEMP = 0.05, 1e-4, 300.0


def _params(noise_mode, seed_key, alpha=ALPHA):
    from magex_gb300 import _lib
    p = _lib.LLGParams()
    p.dt = DT
    p.alpha = alpha
    p.alpha_site = None
    p.precession = 1
    p.integrator = _lib.HEUN
    p.noise = noise_mode
    p.seed = seed_key
    return p


def _sigma_sub(sc):
    from magex_gb300.constants import GAMMA, K_B, MU_B
    return np.ascontiguousarray(np.sqrt(2.0 * ALPHA * K_B * TEMP / (GAMMA * sc.mu_sub * MU_B * DT)), np.float64)


def _noalloc_step(model, params, sigma, lat, noise, step):
    from magex_gb300 import _lib
    from magex_gb300.device import stream_ptr
    _lib.check(model.lib.mgx_llg_step_noalloc(
        model.handle, C.byref(params), _lib.dptr(sigma), C.c_void_p(lat.data_ptr()),
        None if noise is None else C.c_void_p(noise.data_ptr()), C.c_uint64(step), stream_ptr()),
        "mgx_llg_step_noalloc")


def test_noalloc_matches_planned_step_host_noise(cuda):
    """Two consecutive calls with the reference's noise stream (host noise) equal the planned step."""
    from magex_gb300 import _lib
    from magex_gb300.llg import GB300LLG
    from magex_gb300.workloads import bcc_two_site
    sc = bcc_two_site(L=8)                                   # 1,024 spins, full tensors + DMI + SIA
    e0 = sc.init_spins("random", seed=4)
    planned = GB300LLG(sc, ALPHA, DT, TEMP, seed=21, noise="host")
    ref1 = planned.step(e0)
    ref2 = planned.step(ref1)
    model = planned.model
    rng = np.random.default_rng(21)                          # the planned solver's noise stream
    noise = [model.to_lattice(rng.normal(size=(sc.N, 3))) for _ in range(2)]
    lat = model.to_lattice(e0)
    params = _params(_lib.NOISE_HOST, 0)
    sigma = _sigma_sub(sc)
    _noalloc_step(model, params, sigma, lat, noise[0], 0)
    out1 = model.from_lattice(lat).cpu().numpy()
    assert np.abs(out1 - ref1).max() <= 1e-12
    # after the first call (which loads the module and looks the array up), further calls change
    # neither the device's free memory nor anything held by torch's caching allocator
    spare = lat.clone()
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    torch_before = (torch.cuda.memory_allocated(), torch.cuda.memory_reserved())
    _noalloc_step(model, params, sigma, spare, noise[1], 1)
    _noalloc_step(model, params, sigma, lat, noise[1], 1)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free_before, "the no-allocation step changed the free device memory"
    assert (torch.cuda.memory_allocated(), torch.cuda.memory_reserved()) == torch_before
    out2 = model.from_lattice(lat).cpu().numpy()
    assert np.abs(out2 - ref2).max() <= 1e-12
    assert torch.equal(spare, lat)


def test_noalloc_matches_planned_step_philox(cuda):
    """Two consecutive calls with in-kernel Philox noise equal the planned step for the same key."""
    from magex_gb300 import _lib
    from magex_gb300.llg import GB300LLG, _philox_key
    from magex_gb300.workloads import bcc_two_site
    sc = bcc_two_site(L=6)
    e0 = sc.init_spins("random", seed=8)
    planned = GB300LLG(sc, ALPHA, DT, TEMP, seed=33)
    ref1 = planned.step(e0)
    ref2 = planned.step(ref1)
    model = planned.model
    lat = model.to_lattice(e0)
    params = _params(_lib.NOISE_PHILOX, _philox_key(33))
    sigma = _sigma_sub(sc)
    _noalloc_step(model, params, sigma, lat, None, 0)
    assert np.abs(model.from_lattice(lat).cpu().numpy() - ref1).max() <= 1e-12
    _noalloc_step(model, params, sigma, lat, None, 1)
    assert np.abs(model.from_lattice(lat).cpu().numpy() - ref2).max() <= 1e-12


def test_noalloc_rejects_oversized_and_per_site_damping(cuda):
    from magex_gb300 import _lib
    from magex_gb300.device import DeviceModel
    from magex_gb300.workloads import bcc_two_site
    big = bcc_two_site(L=52)                                 # 281,216 sites > the static scratch
    assert big.N > _lib.NOALLOC_MAX_SITES
    model = DeviceModel(big)
    lat = torch.zeros((3, big.N), dtype=torch.float64, device=model.device)
    with pytest.raises(ValueError, match="MGX_NOALLOC_MAX_SITES"):
        _noalloc_step(model, _params(_lib.NOISE_NONE, 0), None, lat, None, 0)
    small = DeviceModel(bcc_two_site(L=4))
    p = _params(_lib.NOISE_NONE, 0)
    al = np.full(small.N, 0.1)
    p.alpha_site = _lib.dptr(al)
    lat = torch.zeros((3, small.N), dtype=torch.float64, device=small.device)
    with pytest.raises(ValueError, match="alpha_site"):
        _noalloc_step(small, p, None, lat, None, 0)


def test_noalloc_follows_reference_trajectory_host_noise(cuda, golden, golden_models):
    """Pinned to the reference directly: the config-2 Hamiltonian (two-site bcc 4^3, full tensors +
    DMI + SIA, B_z = 0.5 T, 300 K) stepped with the reference's own noise stream
    (default_rng(seed).normal per step, magex/llg.py:106-122) through 20 consecutive calls equals
    magex's LLGSolver trajectory after 1 and 20 steps."""
    from helpers import golden_supercell
    from magex_gb300 import _lib
    from magex_gb300.device import DeviceModel
    from magex_gb300.constants import GAMMA, K_B, MU_B
    sc, meta = golden_supercell(golden_models, "bcc2_thermal")
    model = DeviceModel(sc)
    rng = np.random.default_rng(meta["seed"])
    lat = model.to_lattice(golden["bcc2_thermal/e0"])
    params = _params(_lib.NOISE_HOST, 0, alpha=meta["alpha"])
    params.dt = meta["dt"]
    sigma = np.ascontiguousarray(np.sqrt(2.0 * meta["alpha"] * K_B * meta["T"] / (GAMMA * sc.mu_sub * MU_B * meta["dt"])))
    for n in range(1, meta["steps"] + 1):
        noise = model.to_lattice(rng.normal(size=(sc.N, 3)))
        _noalloc_step(model, params, sigma, lat, noise, n - 1)
        if n in meta["keep"]:
            got = model.from_lattice(lat).cpu().numpy()
            assert np.abs(got - golden[f"bcc2_thermal/e{n}"]).max() <= 1e-12 * n, n


@pytest.mark.parametrize("tag", ["sc_cubic", "tri_cubic_thermal"])
def test_noalloc_higher_onsite_terms_follow_reference(cuda, golden, golden_models, tag):
    """Cubic (Kc, rotated axes) and higher uniaxial (K2, K3) anisotropy are stepped as in the planned
    step: the reference's trajectories (Heun at T = 0; Depondt at 5 K with its noise stream)."""
    from helpers import golden_supercell
    from magex_gb300 import _lib
    from magex_gb300.device import DeviceModel
    from magex_gb300.constants import GAMMA, K_B, MU_B
    sc, meta = golden_supercell(golden_models, tag)
    model = DeviceModel(sc)
    thermal = meta["T"] > 0
    rng = np.random.default_rng(meta["seed"])
    lat = model.to_lattice(golden[f"{tag}/e0"])
    params = _params(_lib.NOISE_HOST if thermal else _lib.NOISE_NONE, 0, alpha=meta["alpha"])
    params.dt = meta["dt"]
    params.integrator = _lib.DEPONDT if meta["integrator"] == "depondt" else _lib.HEUN
    sigma = np.ascontiguousarray(np.sqrt(2.0 * meta["alpha"] * K_B * meta["T"] / (GAMMA * sc.mu_sub * MU_B * meta["dt"])))
    for n in range(1, meta["steps"] + 1):
        noise = model.to_lattice(rng.normal(size=(sc.N, 3))) if thermal else None
        _noalloc_step(model, params, sigma if thermal else None, lat, noise, n - 1)
        if n in meta["keep"]:
            got = model.from_lattice(lat).cpu().numpy()
            assert np.abs(got - golden[f"{tag}/e{n}"]).max() <= 1e-12 * n, (tag, n)


def test_noalloc_rejects_per_site_moments_with_noise_and_bad_numbers(cuda):
    """A model whose moments differ site by site has per-site thermal amplitudes, which the
    per-sublattice sigma_sub cannot carry: refused with noise, stepped without.  Non-finite dt,
    negative or non-finite alpha and bad amplitudes are refused as by the planned path."""
    from magex_gb300 import _lib
    from magex_gb300.device import DeviceModel
    from magex_gb300.llg import GB300LLG
    from magex_gb300.workloads import bcc_two_site
    sc = bcc_two_site(L=4)
    sc.mu_site = sc.mu * (1.0 + 0.1 * np.random.default_rng(3).random(sc.N))
    model = DeviceModel(sc)
    e0 = sc.init_spins("random", seed=2)
    lat = model.to_lattice(e0)
    sigma = _sigma_sub(sc)
    with pytest.raises(NotImplementedError, match="moments differ"):
        _noalloc_step(model, _params(_lib.NOISE_PHILOX, 1), sigma, lat, None, 0)
    # without noise the per-site moments enter the field as in the planned step
    planned = GB300LLG(sc, ALPHA, DT, 0.0, seed=1)
    ref = planned.step(planned.step(e0))
    for k in range(2):
        _noalloc_step(model, _params(_lib.NOISE_NONE, 0), None, lat, None, k)
    assert np.abs(model.from_lattice(lat).cpu().numpy() - ref).max() <= 1e-12
    small = DeviceModel(bcc_two_site(L=4))
    lat = small.to_lattice(e0)
    for bad in (float("nan"), float("inf"), -1.0):
        p = _params(_lib.NOISE_NONE, 0)
        p.dt = bad
        with pytest.raises(ValueError, match="dt"):
            _noalloc_step(small, p, None, lat, None, 0)
        with pytest.raises(ValueError, match="alpha"):
            _noalloc_step(small, _params(_lib.NOISE_NONE, 0, alpha=bad), None, lat, None, 0)
        with pytest.raises(ValueError, match="sigma_sub"):
            _noalloc_step(small, _params(_lib.NOISE_PHILOX, 1), np.full(2, bad), lat, None, 0)
