"""mgx_llg_step_noalloc: the Heun step for callers that cannot allocate GPU memory.

Such callers (a framework that owns all device memory through its own pool, a step loop being
captured into a CUDA graph in global mode, a real-time loop) get a step whose scratch lives in a
fixed static device array.  These tests call it through the C ABI and compare it with the planned
entry point (mgx_llg_create + mgx_llg_step, via GB300LLG) on the same spins and the same noise, for
two calls in a row, to the 1e-12 tolerance of the other GPU tests.  The file is named so that pytest
collects it last.
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
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    _noalloc_step(model, params, sigma, lat, noise[1], 1)
    torch.cuda.synchronize()
    free_after = torch.cuda.mem_get_info()[0]
    out2 = model.from_lattice(lat).cpu().numpy()
    assert np.abs(out2 - ref2).max() <= 1e-12
    assert free_after == free_before, "the no-allocation step changed the free device memory"


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
