"""ctypes binding of libmgx.so (declarations in include/mgx.h).

The library is loaded from this package directory only (it is built in-tree by
``magex_gb300.build``).  There is no fallback: if the library is missing or cannot load, every
GPU entry point raises, so a run can never silently fall back to CPU code.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmgx.so")

MGX_OK, MGX_ERR_INVALID, MGX_ERR_UNSUPPORTED, MGX_ERR_CUDA, MGX_ERR_NOMEM = 0, 1, 2, 3, 4
HEUN, DEPONDT = 0, 1
NOISE_NONE, NOISE_HOST, NOISE_PHILOX = 0, 1, 2
PRECISION_FP64, PRECISION_DF32_GATHER, PRECISION_INT48_GATHER, PRECISION_FP64_FIXED_GATHER = 0, 1, 2, 3
MAX_SUBLATTICES = 16
MAX_BONDS = 256
NOALLOC_MAX_SITES = 262144
MC_GAUSSIAN, MC_UNIFORM, MC_HEATBATH, MC_HINZKE = 0, 1, 2, 3
MC_RNG_PHILOX, MC_RNG_HOST = 0, 1

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)
_u8p = C.POINTER(C.c_uint8)


class LatticeDesc(C.Structure):
    _fields_ = [("ns", C.c_int32), ("L", C.c_int32 * 3), ("pbc", C.c_int32 * 3), ("nbond", C.c_int32),
                ("bond_src", _ip), ("bond_dst", _ip), ("bond_R", _ip), ("width", C.c_int32),
                ("bond_table", _dp), ("A_sub", _dp), ("mu_sub", _dp), ("sign_sub", _dp),
                ("B", C.c_double * 3)]


class SiteDesc(C.Structure):
    _fields_ = [("A_site", _dp), ("mu_site", _dp), ("pinned", _u8p)]


class LLGParams(C.Structure):
    _fields_ = [("dt", C.c_double), ("alpha", C.c_double), ("alpha_site", _dp), ("precession", C.c_int32),
                ("integrator", C.c_int32), ("noise", C.c_int32), ("seed", C.c_uint64), ("precision", C.c_int32)]


class CSRDesc(C.Structure):
    _fields_ = [("nsites", C.c_int64), ("ptr", C.POINTER(C.c_int64)), ("nbr", _ip), ("typ", _ip),
                ("ntypes", C.c_int32), ("width", C.c_int32), ("table", _dp), ("A_site", _dp), ("mu_site", _dp),
                ("sign_site", _dp), ("pinned", _u8p), ("B", C.c_double * 3)]


class MCParams(C.Structure):
    _fields_ = [("move", C.c_int32), ("overrelax", C.c_int32), ("rng", C.c_int32), ("sigma", C.c_double),
                ("seed", C.c_uint64), ("precision", C.c_int32)]


#: every exported entry point with (restype, argtypes); the CPU tests check the export list against
#: include/mgx.h
SIGNATURES = {
    "mgx_version": (C.c_int32, []),
    "mgx_last_error": (None, [C.c_char_p, C.c_size_t]),
    "mgx_model_create": (C.c_int32, [C.POINTER(LatticeDesc), C.POINTER(SiteDesc), C.POINTER(C.c_void_p)]),
    "mgx_model_destroy": (C.c_int32, [C.c_void_p]),
    "mgx_model_create_csr": (C.c_int32, [C.POINTER(CSRDesc), C.POINTER(C.c_void_p)]),
    "mgx_model_set_field": (C.c_int32, [C.c_void_p, _dp]),
    "mgx_model_nsites": (C.c_int64, [C.c_void_p]),
    "mgx_model_set_partition": (C.c_int32, [C.c_void_p, C.c_int64, C.c_int32, C.c_int32]),
    "mgx_lattice_layers": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_int32,
                                       C.c_void_p]),
    "mgx_llg_predicted": (C.c_int32, [C.c_void_p, C.POINTER(C.c_void_p)]),
    "mgx_llg_predicted_split": (C.c_int32, [C.c_void_p, C.POINTER(C.c_void_p)]),
    "mgx_pack_spins": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "mgx_unpack_spins": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "mgx_llg_create": (C.c_int32, [C.c_void_p, C.POINTER(LLGParams), C.POINTER(C.c_void_p)]),
    "mgx_llg_destroy": (C.c_int32, [C.c_void_p]),
    "mgx_llg_set_sigma": (C.c_int32, [C.c_void_p, _dp, _dp]),
    "mgx_llg_set_extra_field": (C.c_int32, [C.c_void_p, C.c_void_p]),
    "mgx_llg_set_sot": (C.c_int32, [C.c_void_p, _dp, C.c_double, C.c_double]),
    "mgx_llg_step": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p]),
    "mgx_llg_run": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_int64, C.c_uint64, C.c_void_p]),
    "mgx_llg_stage": (C.c_int32, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p]),
    "mgx_llg_step_host": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p]),
    "mgx_measure_fp64_peak": (C.c_int32, [C.POINTER(C.c_double)]),
    "mgx_write_xyz": (C.c_int32, [C.c_char_p, C.c_int64, _dp, _dp, _dp, _ip, C.POINTER(C.c_char_p), C.c_int32,
                                  C.c_char_p, C.c_int32]),
    "mgx_write_vtk": (C.c_int32, [C.c_char_p, C.c_int64, _dp, _dp, _dp, C.POINTER(C.c_char_p), C.c_int32]),
    "mgx_write_ovf": (C.c_int32, [C.c_char_p, C.c_int64, _dp, _dp]),
    "mgx_write_csv": (C.c_int32, [C.c_char_p, C.c_int64, C.c_int32, _dp, C.c_char_p, C.c_char_p]),
    "mgx_fourier_create": (C.c_int32, [C.c_void_p, C.c_int32, _dp, _dp, C.POINTER(C.c_void_p)]),
    "mgx_fourier_project": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "mgx_fourier_destroy": (C.c_int32, [C.c_void_p]),
    "mgx_colour_stencil": (C.c_int32, [C.POINTER(LatticeDesc), _ip, _ip]),
    "mgx_colour_graph": (C.c_int32, [C.c_int64, C.POINTER(C.c_int64), _ip, _ip, _ip]),
    "mgx_mc_create": (C.c_int32, [C.c_void_p, C.POINTER(MCParams), C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                  C.c_int32, C.POINTER(C.c_void_p)]),
    "mgx_mc_destroy": (C.c_int32, [C.c_void_p]),
    "mgx_mc_set_beta": (C.c_int32, [C.c_void_p, _dp, _dp]),
    "mgx_mc_set_sigma": (C.c_int32, [C.c_void_p, C.c_double]),
    "mgx_mc_host_draws": (C.c_int32, [C.c_void_p, C.POINTER(C.c_int64)]),
    "mgx_mc_sweep": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]),
    "mgx_mc_counts": (C.c_int32, [C.c_void_p, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64), C.c_int32,
                                  C.c_void_p]),
    "mgx_mc_set_chains": (C.c_int32, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p]),
    "mgx_mc_chain_counts": (C.c_int32, [C.c_void_p, C.c_void_p, C.POINTER(C.c_uint64), C.c_void_p, C.c_int32,
                                         C.c_void_p]),
    "mgx_mc_adapt_sigma": (C.c_int32, [C.c_void_p, C.c_void_p]),
    "mgx_llg_step_noalloc": (C.c_int32, [C.c_void_p, C.POINTER(LLGParams), _dp, C.c_void_p, C.c_void_p, C.c_uint64,
                                         C.c_void_p]),
    "mgx_batch_create": (C.c_int32, [C.POINTER(C.c_void_p), C.POINTER(LLGParams), C.c_int32, C.POINTER(C.c_void_p)]),
    "mgx_batch_destroy": (C.c_int32, [C.c_void_p]),
    "mgx_batch_nsites": (C.c_int64, [C.c_void_p]),
    "mgx_batch_offset": (C.c_int64, [C.c_void_p, C.c_int32]),
    "mgx_batch_set_sigma": (C.c_int32, [C.c_void_p, C.c_int32, _dp]),
    "mgx_batch_sync_models": (C.c_int32, [C.c_void_p]),
    "mgx_batch_set_launch": (C.c_int32, [C.c_void_p, C.c_int32, C.c_int32]),
    "mgx_batch_step": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p]),
    "mgx_batch_run": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_int64, C.c_uint64, C.c_int32, C.c_void_p]),
    "mgx_batch_observables": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "mgx_batch_set_triangles": (C.c_int32, [C.c_void_p, _ip, _dp, C.POINTER(C.c_int64)]),
    "mgx_batch_topological_charge": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "mgx_model_set_couplings": (C.c_int32, [C.c_void_p, _dp]),
    "mgx_model_set_onsite": (C.c_int32, [C.c_void_p, _dp]),
    "mgx_model_set_onsite_higher": (C.c_int32, [C.c_void_p, _dp, _dp, _dp, _dp, _dp]),
    "mgx_adjoint_create": (C.c_int32, [C.c_void_p, C.c_void_p, _ip, _ip, C.c_int32, C.POINTER(LLGParams), C.c_int32,
                                       C.POINTER(C.c_void_p)]),
    "mgx_adjoint_destroy": (C.c_int32, [C.c_void_p]),
    "mgx_adjoint_set_sigma": (C.c_int32, [C.c_void_p, _dp]),
    "mgx_adjoint_sync_models": (C.c_int32, [C.c_void_p]),
    "mgx_adjoint_forward": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_int32, C.c_uint64, C.c_void_p, C.c_void_p]),
    "mgx_adjoint_backward": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p]),
    "mgx_adjoint_storage_doubles": (C.c_int64, [C.c_void_p]),
    "mgx_adjoint_set_storage": (C.c_int32, [C.c_void_p, C.c_void_p]),
    "mgx_adjoint_zero_grads": (C.c_int32, [C.c_void_p, C.c_void_p]),
    "mgx_adjoint_grads": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "mgx_adjoint_grads_onsite_higher": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "mgx_adjoint_set_needs": (C.c_int32, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32]),
    "mgx_adjoint_select_own_storage": (C.c_int32, [C.c_void_p, C.c_int32]),
    "mgx_observables": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "mgx_observables_n": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p]),
    "mgx_effective_field": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "mgx_topological_charge": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64,
                                           C.c_void_p, C.c_void_p]),
}

_lib = None


def load(path=LIB_PATH):
    """Load libmgx.so and attach signatures (cached).  Raises RuntimeError if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"libmgx.so not found at {path}: build it with `python -m magex_gb300.build` "
                           "(the GB300 LLG path has no CPU fallback)")
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def last_error():
    buf = C.create_string_buffer(1024)
    load().mgx_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def check(status, what=""):
    """Map an mgx_status to the exception magex raises in the same situation."""
    if status == MGX_OK:
        return
    msg = f"{what}: {last_error()}" if what else last_error()
    if status == MGX_ERR_INVALID:
        raise ValueError(msg)
    if status == MGX_ERR_UNSUPPORTED:
        raise NotImplementedError(msg)
    if status == MGX_ERR_NOMEM:
        raise MemoryError(msg)
    raise RuntimeError(msg)


def dptr(a):
    """ctypes double* of a C-contiguous float64 numpy array (or None)."""
    if a is None:
        return None
    return a.ctypes.data_as(_dp)


def iptr(a):
    return None if a is None else a.ctypes.data_as(_ip)


def u8ptr(a):
    return None if a is None else a.ctypes.data_as(_u8p)
