"""lqt1_gb300 -- GB300-native (sm_103a) monodomain TPORd simulator.

A drop-in for the hot path of ShugangZhang/LQT1: the TPORd cell model
(SingleCell/TPORd.cc) with the 1D/2D/3D tissue stepping of OneD.cc,
new_11.cu and GPU3D.cu, as hand-written CUDA kernels behind the C ABI in
include/lqt.h.  This package is the Python side of that ABI.
"""
from ._native import (EMPTY, ENDO, EPI, FP64, LVENDO, LVEPI, MCELL, MIXED, LqtError, Model,  # noqa: F401
                      lib, model)
from .batch import Batch, InstanceSpec, OneDStrand, oned_types  # noqa: F401
from .cell import STATE_NAMES, TPORdCells, initial_state  # noqa: F401

__all__ = ["TPORdCells", "Batch", "InstanceSpec", "OneDStrand", "oned_types", "initial_state", "model", "lib",
           "Model", "LqtError", "FP64", "MIXED", "LVEPI", "LVENDO", "EPI", "ENDO", "MCELL", "EMPTY", "STATE_NAMES"]
from . import batch, geometry  # noqa: E402,F401
from .sim import Sim  # noqa: E402,F401

__all__ += ["Sim", "geometry"]


def __getattr__(name):
    # protocols, surrogate, replicas load on first use (and run as
    # `python -m lqt1_gb300.<module>` without a second import)
    if name in ("protocols", "surrogate", "replicas"):
        import importlib
        return importlib.import_module("." + name, __name__)
    raise AttributeError(name)
