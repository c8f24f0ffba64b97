"""magex_gb300 -- GB300-native (sm_103a) stochastic LLG step for magex spin models.

Public API (drop-in for the magex LLG path):
  LLGSolver / GB300LLG       magex.llg.LLGSolver (heun, depondt) on one GB300
  Supercell                  supercell of a UnitCellModel without the 3N x 3N matrix
  load_results, make_model   magex results.json loader and textbook-model builder
  UnitCellModel, constants   MU_B, K_B, GAMMA
  MetropolisMC, point, points, parallel_tempering, estimate_tc
                             magex.montecarlo / magex.advanced_mc colour-sweep Monte Carlo (mc.py)
  BatchedLLG, AdjointLLG, structure_factor, the writers of output.py: batched.py, adjoint.py,
                             spectra.py, output.py
"""
from .constants import GAMMA, K_B, MU_B
from .lattice import Supercell
from .spinmodel import UnitCellModel, load_results, make_model, normalize, write_model

__all__ = ["GAMMA", "K_B", "MU_B", "Supercell", "UnitCellModel", "load_results", "make_model", "normalize",
           "write_model", "LLGSolver", "GB300LLG", "DeviceModel", "MetropolisMC", "point", "points",
           "parallel_tempering", "estimate_tc"]


def __getattr__(name):
    # torch-dependent modules load on first use, so the host-side model code imports without torch
    if name in ("LLGSolver", "GB300LLG"):
        from . import llg
        return getattr(llg, name)
    if name in ("MetropolisMC", "point", "points", "parallel_tempering", "estimate_tc"):
        from . import mc
        return getattr(mc, name)
    if name == "DeviceModel":
        from .device import DeviceModel
        return DeviceModel
    raise AttributeError(name)
