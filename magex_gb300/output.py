"""Spin and table outputs at scale: magex's writers (magex/observables.py:122-161, magex/llg.py:286-297)
with the text formatted natively in parallel (``mgx_write_*``), byte-for-byte the same files.

    write_xyz(path, system, e)           extended XYZ for OVITO / ASE
    write_vtk(path, system, e, extra)    VTK legacy polydata for ParaView
    write_ovf_atomistic(path, system, e) OVF 2.0 irregular mesh
    save_spins(path, system, e)          .npz (numpy) + .csv of positions and spins
    write_table(path, table)             LLGSolver.run table as CSV

``e`` may be a numpy array or a torch tensor (CUDA tensors are copied to the host once).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib


def _host(e):
    try:
        import torch
        if isinstance(e, torch.Tensor):
            return np.ascontiguousarray(e.detach().cpu().numpy(), np.float64)
    except ImportError:
        pass
    return np.ascontiguousarray(e, np.float64)


def _material(system):
    m = getattr(system, "material", None)
    return np.zeros(system.N, int) if m is None else np.asarray(m)


def write_xyz(path, system, e, comment="", append=False):
    """Extended XYZ: species, position, spin vector, moment per site (magex/observables.py:122-132)."""
    lib = _lib.load()
    e = _host(e)
    pos = np.ascontiguousarray(system.positions, np.float64)
    mu = np.ascontiguousarray(np.broadcast_to(np.asarray(system.mu, float), (system.N,)), np.float64)
    sub = np.ascontiguousarray(system.sublattice, np.int32)
    names = [str(s).encode() for s in system.uc.symbols]
    arr = (C.c_char_p * len(names))(*names)
    _lib.check(lib.mgx_write_xyz(str(path).encode(), system.N, _lib.dptr(pos), _lib.dptr(e), _lib.dptr(mu),
                                 _lib.iptr(sub), arr, len(names), str(comment).encode(), int(bool(append))),
               "mgx_write_xyz")
    return path


def write_vtk(path, system, e, extra=None):
    """VTK legacy polydata with spin vectors and the scalars mz, sublattice, material and any extra
    per-site arrays (magex/observables.py:135-150)."""
    lib = _lib.load()
    e = _host(e)
    N = system.N
    items = [("mz", e[:, 2]), ("sublattice", system.sublattice), ("material", _material(system))] + \
        list((extra or {}).items())
    sc = np.ascontiguousarray(np.stack([np.asarray(a, float).reshape(N) for _, a in items]), np.float64)
    names = [str(k).encode() for k, _ in items]
    arr = (C.c_char_p * len(names))(*names)
    pos = np.ascontiguousarray(system.positions, np.float64)
    _lib.check(lib.mgx_write_vtk(str(path).encode(), N, _lib.dptr(pos), _lib.dptr(e), _lib.dptr(sc), arr,
                                 len(names)), "mgx_write_vtk")
    return path


def write_ovf_atomistic(path, system, e):
    """OVF 2.0 irregular-mesh text file (magex/observables.py:153-161)."""
    lib = _lib.load()
    e = _host(e)
    pos = np.ascontiguousarray(system.positions, np.float64)
    _lib.check(lib.mgx_write_ovf(str(path).encode(), system.N, _lib.dptr(pos), _lib.dptr(e)), "mgx_write_ovf")
    return path


def write_table(path, table):
    """LLGSolver.run table as CSV (magex/llg.py:287-289)."""
    lib = _lib.load()
    t = np.ascontiguousarray(np.atleast_2d(np.asarray(table, float)), np.float64)
    _lib.check(lib.mgx_write_csv(str(path).encode(), t.shape[0], t.shape[1], _lib.dptr(t), b"%.8g",
                                 b"t_ps,E_per_spin_meV,mx,my,mz,order_parameter,max_torque_T"), "mgx_write_csv")
    return path


def save_spins(path, system, e):
    """Spins with positions, moments, sublattices and the cell as .npz, and positions + spins as .csv
    next to it (magex/llg.py:292-297)."""
    lib = _lib.load()
    e = _host(e)
    np.savez_compressed(path, spins=e, positions=system.positions, mu=system.mu, sublattice=system.sublattice,
                        cell=system.uc.cell, supercell=np.array(system.L))
    rows = np.ascontiguousarray(np.column_stack([system.positions, e]), np.float64)
    csv = str(path).replace(".npz", ".csv")
    _lib.check(lib.mgx_write_csv(csv.encode(), rows.shape[0], 6, _lib.dptr(rows), b"%.6f", b"x_A,y_A,z_A,ex,ey,ez"),
               "mgx_write_csv")
    return path
